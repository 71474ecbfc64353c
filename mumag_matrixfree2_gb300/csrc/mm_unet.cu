// Learned demag warm start: a 3D U-Net over a voxel grid, trained and run on the GPU by this
// file's own kernels.
//
//  * Convolutions (3x3x3, stride 1, zero padding 1) are implicit GEMMs on the 5th-generation tensor
//    cores: BF16 operands staged in shared memory by bulk copies, tcgen05.mma issued by one thread,
//    FP32 accumulators in TMEM, read back with tcgen05.ld for the epilogue (bias, ReLU, halo zero,
//    BF16 store).  The backward-data pass is the same kernel with the mirrored, transposed weights.
//  * Activation layout: every tensor of a G^3 level is stored zero-padded to P^3 (P = G + 2) and
//    flattened; channels are grouped in 8-channel chunk planes, 16 bytes per voxel, each plane with
//    zero guard voxels on both sides.  A tap (dz, dy, dx) of the convolution is then a pure shift of
//    the flat index by dz P^2 + dy P + dx, so the A operand of every tap is a contiguous run of rows
//    of one staged window: the descriptors differ only in their start address.  Halo outputs are
//    computed and stored as zero, which keeps the padding invariant for the next layer.
//  * Weight gradients reduce over voxels (K = voxels, M = input channels can be 16): they use
//    warp-level mma.sync (m16n8k16, BF16 in, FP32 accumulate) with ldmatrix.trans staging, split
//    over voxel ranges into per-block partials summed in a fixed order (deterministic).
//  * Everything else (pooling, upsampling with skip addition, ReLU masks, the loss, Adam, the BF16
//    weight copies, mesh <-> grid transfers) is plain elementwise CUDA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mumag_cuda.h"
#include "mm_tc.cuh"

namespace mmn {

// ------------------------------------------------------------------------------------------------
// geometry of one level
// ------------------------------------------------------------------------------------------------
constexpr int MT = 2;        // 128-row M tiles per CTA of the convolution
constexpr int MT_MAX = 4;    // guard sizing
struct Vol {
  int G, P, S;    // interior edge, padded edge, P^3
  int guard;      // zero voxels before and after every chunk plane
  int plane;      // voxels per chunk plane (guard + S + guard)
  int t0, t1;     // computed output range of the flat index: the interior z planes [P^2, P^2 (P-1))
};
inline Vol make_vol(int G) {
  Vol v;
  v.G = G;
  v.P = G + 2;
  v.S = v.P * v.P * v.P;
  v.guard = ((128 * MT_MAX + v.P + 1) + 7) / 8 * 8;
  v.plane = v.guard + v.S + v.guard;
  v.t0 = v.P * v.P;
  v.t1 = v.P * v.P * (v.P - 1);
  return v;
}

__device__ __forceinline__ bool interior(const Vol& v, int p) {
  const int PP = v.P * v.P;
  const int z = p / PP;
  const int r = p - z * PP;
  const int y = r / v.P;
  const int x = r - y * v.P;
  return z >= 1 && z <= v.G && y >= 1 && y <= v.G && x >= 1 && x <= v.G;
}
// flat padded index of interior voxel (z, y, x) (0-based interior coordinates)
__device__ __forceinline__ int flat(const Vol& v, int z, int y, int x) { return ((z + 1) * v.P + (y + 1)) * v.P + x + 1; }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ void unpack8(const uint4& q, float (&f)[8]) {
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f[2 * i] = __uint_as_float(w[i] << 16);
    f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
  }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  return make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
}

// ------------------------------------------------------------------------------------------------
// tcgen05 convolution
// ------------------------------------------------------------------------------------------------
struct ConvArgs {
  const uint4* in;   // input activations, cin / 8 chunk planes per sample
  const uint4* wk;   // weights [cout/NT][cin/16][27][2][NT][8] bf16
  const float* bias; // cout, or null
  uint4* out;        // output activations, cout / 8 chunk planes per sample
  Vol v;
  int cin, cout;
  int relu;
  int* err;          // set to 1 when a wait gave up
};

// Shared memory of one CTA: barriers, then NST stages of A windows (3 dz x 2 chunks x WL rows) and
// B weights (27 taps x 2 chunks x NT rows), 16 bytes per row.
__host__ __device__ inline int conv_wl(int P) { return 128 * MT + 2 * P + 2; }
__host__ __device__ inline size_t conv_smem(int P, int cin, int NT) {
  const int nst = cin >= 32 ? 2 : 1;
  return 1024 + (size_t)nst * ((size_t)6 * conv_wl(P) * 16 + (size_t)54 * NT * 16);
}

template <int CIN, int NT>
__global__ void __launch_bounds__(128) k_conv_tc(ConvArgs a) {
  constexpr int NCP = CIN / 16;           // K stages: 16 input channels each
  constexpr int NST = NCP >= 2 ? 2 : 1;   // stage buffers
  constexpr uint32_t NCOL = (MT * NT <= 32) ? 32 : (MT * NT <= 64 ? 64 : (MT * NT <= 128 ? 128 : 256));
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);      // [NST]
  uint64_t* done = full + 2;                                // [NST]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 64);
  int* s_fail = reinterpret_cast<int*>(smem + 68);
  const Vol v = a.v;
  const int P = v.P;
  const int WL = conv_wl(P);
  unsigned char* Abuf = smem + 1024;
  const size_t Astage = (size_t)6 * WL * 16;
  const size_t Bstage = (size_t)54 * NT * 16;
  unsigned char* Bbuf = Abuf + NST * Astage;

  const int tile0 = v.t0 + blockIdx.x * (128 * MT);
  const int cot = blockIdx.y;
  const int b = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) mtc::tmem_alloc(tslot, NCOL);
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mtc::mbar_init(&full[s], 1);
      mtc::mbar_init(&done[s], 1);
    }
    *s_fail = 0;
    mtc::fence_mbar_init();
  }
  mtc::tc_fence_before();
  __syncthreads();
  mtc::tc_fence_after();
  const uint32_t tbase = *tslot;

  if (threadIdx.x == 0) {
    const size_t in_plane0 = (size_t)b * (CIN / 8);
    auto issue = [&](int cp, int st) {
      unsigned char* A = Abuf + st * Astage;
      unsigned char* B = Bbuf + st * Bstage;
      mtc::mbar_expect_tx(&full[st], (uint32_t)(Astage + Bstage));
#pragma unroll
      for (int dz = 0; dz < 3; ++dz)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const size_t plane = in_plane0 + 2 * cp + h;
          const long long start = (long long)v.guard + tile0 + (dz - 1) * P * P - (P + 1);
          mtc::bulk_g2s(A + (size_t)(dz * 2 + h) * WL * 16, a.in + plane * v.plane + start, (uint32_t)WL * 16,
                        &full[st]);
        }
      mtc::bulk_g2s(B, a.wk + ((size_t)cot * NCP + cp) * 54 * NT, (uint32_t)Bstage, &full[st]);
    };
    // bookkeeping for the failure path: chunks whose copies were issued / seen complete, the last
    // chunk whose MMAs were committed and whether their completion was seen
    int issued = 0, loaded = 0, committed = -1;
    bool mma_seen = true;
    for (int s = 0; s < NST && s < NCP; ++s, ++issued) issue(s, s);
    constexpr uint32_t IDESC = mtc::idesc_bf16(128, NT);
    bool ok = true;
    for (int cp = 0; cp < NCP && ok; ++cp) {
      const int st = cp % NST;
      const uint32_t par = (uint32_t)(cp / NST) & 1u;
      if (!mtc::mbar_wait(&full[st], par)) {
        ok = false;
        break;
      }
      loaded = cp + 1;
      mtc::tc_fence_after();
      const uint32_t As = mtc::smem_u32(Abuf + st * Astage);
      const uint32_t Bs = mtc::smem_u32(Bbuf + st * Bstage);
#pragma unroll 1
      for (int t = 0; t < 27; ++t) {
        const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;  // shifts + 1
        const uint64_t bd = mtc::sdesc(Bs + (uint32_t)(t * 2 * NT * 16), NT * 16, 128);
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
          const uint32_t aoff = (uint32_t)((dz * 2 * WL + mt * 128 + dy * P + dx) * 16);
          const uint64_t ad = mtc::sdesc(As + aoff, (uint32_t)WL * 16, 128);
          mtc::mma_bf16(tbase + (uint32_t)(mt * NT), ad, bd, IDESC, cp > 0 || t > 0);
        }
      }
      mtc::mma_commit(&done[st]);
      committed = cp;
      mma_seen = false;
      if (cp + NST < NCP) {
        if (!mtc::mbar_wait(&done[st], par)) {
          ok = false;
          break;
        }
        mma_seen = true;  // a commit's arrival covers every earlier MMA of this thread
        issue(cp + NST, st);
        ++issued;
      }
    }
    if (!ok) {
      // A wait gave up: raise the (sticky) error flag, then drain before the tensor memory and the
      // shared-memory stages are released: the MMAs committed last, then every copy still in flight,
      // each wait bounded like the others.  If a drain wait gives up too, the memory is released
      // with that work outstanding; the flag has already made every result of this launch, and
      // every later call of the network, an error.
      *s_fail = 1;
      atomicExch(a.err, 1);
      if (committed >= 0 && !mma_seen) mtc::mbar_wait(&done[committed % NST], (uint32_t)(committed / NST) & 1u);
      for (int c = loaded; c < issued; ++c) mtc::mbar_wait(&full[c % NST], (uint32_t)(c / NST) & 1u);
    }
  }
  __syncthreads();
  if (*s_fail == 0) {
    const int last = NCP - 1;
    if (!mtc::mbar_wait(&done[last % NST], (uint32_t)(last / NST) & 1u)) {
      atomicExch(a.err, 1);
    } else {
      mtc::tc_fence_after();
      const int row = warp * 32 + lane;
      const size_t out_plane0 = (size_t)b * (a.cout / 8);
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        const int p = tile0 + mt * 128 + row;
        const bool in = interior(v, p);
#pragma unroll
        for (int c16 = 0; c16 < NT / 16; ++c16) {
          float acc[16];
          mtc::tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mt * NT + c16 * 16), acc);
          const int co0 = cot * NT + c16 * 16;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float y = acc[j] + (a.bias ? __ldg(a.bias + co0 + j) : 0.0f);
            if (a.relu) y = fmaxf(y, 0.0f);
            acc[j] = in ? y : 0.0f;
          }
          float lo[8], hi[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            lo[j] = acc[j];
            hi[j] = acc[8 + j];
          }
          a.out[(out_plane0 + co0 / 8) * v.plane + v.guard + p] = pack8(lo);
          a.out[(out_plane0 + co0 / 8 + 1) * v.plane + v.guard + p] = pack8(hi);
        }
      }
    }
  }
  mtc::tc_fence_before();
  __syncthreads();
  if (warp == 0) mtc::tmem_dealloc(tbase, NCOL);
}

// ------------------------------------------------------------------------------------------------
// weight gradient (mma.sync m16n8k16, BF16 in, FP32 accumulate), split over voxel ranges
// ------------------------------------------------------------------------------------------------
struct WgArgs {
  const uint4* x;   // layer input, cin / 8 chunk planes per sample
  const uint4* d;   // gradient of the pre-activation output, cout / 8 chunk planes per sample
  float* part;      // [batch][nsplit][27][cin][cout]
  Vol v;
  int cin, cout;
  int vpb;          // voxels per block (multiple of 64)
  int nsplit;
};

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t addr, uint32_t& r0, uint32_t& r1) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(addr));
}
__device__ __forceinline__ void mma_16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                          uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int CIT, int COT>
__global__ void __launch_bounds__(128) k_wgrad(WgArgs a) {
  constexpr int MTL = CIT / 16, NTL = COT / 8, TILES = MTL * NTL, TPW = (TILES + 3) / 4;
  __shared__ __align__(16) uint4 Xs[CIT / 8][64];
  __shared__ __align__(16) uint4 Ds[COT / 8][64];
  const Vol v = a.v;
  const int split = blockIdx.x;
  int yy = blockIdx.y;
  const int nct = a.cout / COT, nit = a.cin / CIT;
  const int cot = yy % nct;
  yy /= nct;
  const int cit = yy % nit;
  const int t = yy / nit;
  const int b = blockIdx.z;
  const int shift = (t / 9 - 1) * v.P * v.P + ((t / 3) % 3 - 1) * v.P + (t % 3 - 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[TPW][4];
#pragma unroll
  for (int q = 0; q < TPW; ++q)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[q][i] = 0.0f;
  const int vbeg = v.t0 + split * a.vpb;
  const int vend = min(v.t1, vbeg + a.vpb);
  const size_t xp0 = (size_t)b * (a.cin / 8) + cit * (CIT / 8);
  const size_t dp0 = (size_t)b * (a.cout / 8) + cot * (COT / 8);
  for (int v0 = vbeg; v0 < vend; v0 += 64) {
    __syncthreads();
    for (int i = threadIdx.x; i < (CIT / 8) * 64; i += 128) {
      const int c = i >> 6, r = i & 63;
      Xs[c][r] = a.x[(xp0 + c) * v.plane + v.guard + v0 + r + shift];
    }
    for (int i = threadIdx.x; i < (COT / 8) * 64; i += 128) {
      const int c = i >> 6, r = i & 63;
      Ds[c][r] = (v0 + r < vend) ? a.d[(dp0 + c) * v.plane + v.guard + v0 + r] : make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
      for (int q = 0; q < TPW; ++q) {
        const int j = warp + 4 * q;
        if (j < TILES) {
          const int mi = j / NTL, ni = j % NTL;
          const int mat = lane >> 3, r = lane & 7;
          const uint32_t aaddr = mtc::smem_u32(&Xs[mi * 2 + (mat & 1)][kk * 16 + (mat >> 1) * 8 + r]);
          uint32_t a0, a1, a2, a3, b0, b1;
          ldsm_x4_t(aaddr, a0, a1, a2, a3);
          const int l16 = lane & 15;
          const uint32_t baddr = mtc::smem_u32(&Ds[ni][kk * 16 + l16]);
          ldsm_x2_t(baddr, b0, b1);
          mma_16816(acc[q], a0, a1, a2, a3, b0, b1);
        }
      }
    }
  }
  float* out = a.part + (((size_t)b * a.nsplit + split) * 27 + t) * (size_t)a.cin * a.cout;
  const int g = lane >> 2, tg = lane & 3;
#pragma unroll
  for (int q = 0; q < TPW; ++q) {
    const int j = warp + 4 * q;
    if (j < TILES) {
      const int mi = j / NTL, ni = j % NTL;
      const int ci = cit * CIT + mi * 16 + g;
      const int co = cot * COT + ni * 8 + 2 * tg;
      out[(size_t)ci * a.cout + co] = acc[q][0];
      out[(size_t)ci * a.cout + co + 1] = acc[q][1];
      out[(size_t)(ci + 8) * a.cout + co] = acc[q][2];
      out[(size_t)(ci + 8) * a.cout + co + 1] = acc[q][3];
    }
  }
}

// dW[i] = sum over (sample, split) of the partials, in order; rows ci >= keep_ci are zeroed
__global__ void k_sum_parts(const float* part, int nparts, int n, int cin, int cout, int keep_ci, float* dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nparts; ++k) s += part[(size_t)k * n + i];
    const int ci = (i / cout) % cin;
    dst[i] = ci < keep_ci ? (float)s : 0.0f;
  }
}

// bias-gradient partials: bpart[(b * nsplit + split) * cout + co] = sum over the split's voxels
__global__ void __launch_bounds__(128) k_bias_part(const uint4* d, Vol v, int cout, int vpb, int nsplit, float* bpart) {
  __shared__ float s[128][8];
  const int split = blockIdx.x, b = blockIdx.y;
  const int nch = cout / 8;
  const int vbeg = v.t0 + split * vpb, vend = min(v.t1, vbeg + vpb);
  for (int c = 0; c < nch; ++c) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint4* pl = d + ((size_t)b * nch + c) * v.plane + v.guard;
    for (int p = vbeg + threadIdx.x; p < vend; p += 128) {
      float f[8];
      unpack8(pl[p], f);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] += f[j];
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) s[threadIdx.x][j] = acc[j];
    __syncthreads();
    if (threadIdx.x < 8) {
      float t = 0.0f;
      for (int i = 0; i < 128; ++i) t += s[i][threadIdx.x];
      bpart[((size_t)b * nsplit + split) * cout + c * 8 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------------
// elementwise kernels (one thread per interior voxel and 8-channel chunk)
// ------------------------------------------------------------------------------------------------
// out (level G/2) = 2x2x2 average of in (level G)
__global__ void k_pool(const uint4* in, Vol vf, uint4* out, Vol vc, int nch, int nb) {
  const int Gc = vc.G;
  const long long n = (long long)nb * nch * Gc * Gc * Gc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int x = r % Gc; r /= Gc;
    const int y = r % Gc; r /= Gc;
    const int z = r % Gc; r /= Gc;
    const long long pl = r;  // sample * nch + chunk
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 8; ++c) {
      float f[8];
      unpack8(in[pl * vf.plane + vf.guard + flat(vf, 2 * z + (c >> 2), 2 * y + ((c >> 1) & 1), 2 * x + (c & 1))], f);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] += f[j];
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] *= 0.125f;
    out[pl * vc.plane + vc.guard + flat(vc, z, y, x)] = pack8(acc);
  }
}

// out (level G) = nearest upsampling of in (level G/2) + skip (level G)
__global__ void k_up_add(const uint4* in, Vol vc, const uint4* skip, uint4* out, Vol vf, int nch, int nb) {
  const int G = vf.G;
  const long long n = (long long)nb * nch * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int x = r % G; r /= G;
    const int y = r % G; r /= G;
    const int z = r % G; r /= G;
    const long long pl = r;
    float a[8], s[8];
    unpack8(in[pl * vc.plane + vc.guard + flat(vc, z >> 1, y >> 1, x >> 1)], a);
    const int pf = flat(vf, z, y, x);
    unpack8(skip[pl * vf.plane + vf.guard + pf], s);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] += s[j];
    out[pl * vf.plane + vf.guard + pf] = pack8(a);
  }
}

// d_fine = d_coarse(parent) / 8 + d_skip
__global__ void k_pool_bwd_add(const uint4* dc, Vol vc, const uint4* dskip, uint4* df, Vol vf, int nch, int nb) {
  const int G = vf.G;
  const long long n = (long long)nb * nch * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int x = r % G; r /= G;
    const int y = r % G; r /= G;
    const int z = r % G; r /= G;
    const long long pl = r;
    float a[8], s[8];
    unpack8(dc[pl * vc.plane + vc.guard + flat(vc, z >> 1, y >> 1, x >> 1)], a);
    const int pf = flat(vf, z, y, x);
    unpack8(dskip[pl * vf.plane + vf.guard + pf], s);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = a[j] * 0.125f + s[j];
    df[pl * vf.plane + vf.guard + pf] = pack8(a);
  }
}

// d_coarse = sum of the 8 children of d_fine
__global__ void k_up_bwd(const uint4* df, Vol vf, uint4* dc, Vol vc, int nch, int nb) {
  const int Gc = vc.G;
  const long long n = (long long)nb * nch * Gc * Gc * Gc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int x = r % Gc; r /= Gc;
    const int y = r % Gc; r /= Gc;
    const int z = r % Gc; r /= Gc;
    const long long pl = r;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 8; ++c) {
      float f[8];
      unpack8(df[pl * vf.plane + vf.guard + flat(vf, 2 * z + (c >> 2), 2 * y + ((c >> 1) & 1), 2 * x + (c & 1))], f);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] += f[j];
    }
    dc[pl * vc.plane + vc.guard + flat(vc, z, y, x)] = pack8(acc);
  }
}

// d <- d * (y > 0) (ReLU backward, in place)
__global__ void k_relu_mask(uint4* d, const uint4* y, Vol v, int nch, int nb) {
  const int G = v.G;
  const long long n = (long long)nb * nch * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int x = r % G; r /= G;
    const int yy = r % G; r /= G;
    const int z = r % G; r /= G;
    const size_t at = (size_t)r * v.plane + v.guard + flat(v, z, yy, x);
    float a[8], m[8];
    unpack8(d[at], a);
    unpack8(y[at], m);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = m[j] > 0.0f ? a[j] : 0.0f;
    d[at] = pack8(a);
  }
}

// FP32 [nb][G^3][4] -> chunk 0 of the input tensor (channels 4..7 zero; chunk 1 stays zero)
__global__ void k_pack_input(const float* src, Vol v, uint4* x, int nb) {
  const int G = v.G;
  const long long n = (long long)nb * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int xx = r % G; r /= G;
    const int y = r % G; r /= G;
    const int z = r % G; r /= G;
    const float* s = src + i * 4;
    float f[8] = {s[0], s[1], s[2], s[3], 0, 0, 0, 0};
    x[(size_t)r * 2 * v.plane + v.guard + flat(v, z, y, xx)] = pack8(f);
  }
}

// all channels of one sample of a tensor -> FP32 [G^3][C]
__global__ void k_read_tensor(const uint4* y, Vol v, int nch, int sample, float* dst) {
  const int G = v.G;
  const long long n = (long long)nch * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % nch);
    long long r = i / nch;
    const int xx = r % G; r /= G;
    const int yy = r % G; r /= G;
    const int z = (int)r;
    float f[8];
    unpack8(y[((size_t)sample * nch + c) * v.plane + v.guard + flat(v, z, yy, xx)], f);
#pragma unroll
    for (int j = 0; j < 8; ++j) dst[(((long long)z * G + yy) * G + xx) * nch * 8 + c * 8 + j] = f[j];
  }
}

// channel 0 of the output -> FP32 [nb][G^3]
__global__ void k_unpack_out(const uint4* y, Vol v, int nch, float* dst, int nb) {
  const int G = v.G;
  const long long n = (long long)nb * G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int xx = r % G; r /= G;
    const int yy = r % G; r /= G;
    const int z = r % G; r /= G;
    float f[8];
    unpack8(y[(size_t)r * nch * v.plane + v.guard + flat(v, z, yy, xx)], f);
    dst[i] = f[0];
  }
}

// Loss: mean over nb * G^3 voxels of (y0 - target)^2; seeds dy (channel 0 = 2 (y0 - t) / n, other
// channels of chunk 0 zero).  Block partials of the squared error (FP64) for a fixed-order host sum.
__global__ void __launch_bounds__(256) k_loss(const uint4* y, Vol v, int nch, const float* target, int nb,
                                               uint4* dy, double* part) {
  __shared__ double s[256];
  const int G = v.G;
  const long long n = (long long)nb * G * G * G;
  const float sc = (float)(2.0 / (double)n);
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int xx = r % G; r /= G;
    const int yy = r % G; r /= G;
    const int z = r % G; r /= G;
    const size_t at = (size_t)r * nch * v.plane + v.guard + flat(v, z, yy, xx);
    float f[8];
    unpack8(y[at], f);
    const float e = f[0] - target[i];
    acc += (double)e * (double)e;
    float g[8] = {sc * e, 0, 0, 0, 0, 0, 0, 0};
    dy[at] = pack8(g);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// BF16 weight copies in the convolution kernel's layout: forward [cout/NT][cin/16][27][2][NT][8] from
// W[t][ci][co]; backward-data (transposed) the same layout for cin' = cout, cout' = cin with
// W'[t][co][ci] = W[26 - t][ci][co].
__global__ void k_prep_weights(const float* w, int cin, int cout, int NT, int transposed, uint4* dst) {
  const int ci_ = transposed ? cout : cin;   // input channels of the kernel being fed
  const int co_ = transposed ? cin : cout;
  const int n = (co_ / NT) * (ci_ / 16) * 54 * NT;  // 16-byte rows
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int r = i;
    const int nn = r % NT; r /= NT;
    const int h = r % 2; r /= 2;
    const int t = r % 27; r /= 27;
    const int cp = r % (ci_ / 16); r /= (ci_ / 16);
    const int cot = r;
    const int co = cot * NT + nn;
    float f[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int ci = (2 * cp + h) * 8 + e;
      f[e] = transposed ? w[((size_t)(26 - t) * cin + co) * cout + ci] : w[((size_t)t * cin + ci) * cout + co];
    }
    dst[i] = pack8(f);
  }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// mesh -> grid: channel c of voxel v = sum_k w[v][k] f_c(node idx[v][k]) * scale_c (4 nodes; idx < 0
// ends the list), written as chunk 0 of sample `sample` (channels 0..2 from a (N,3) field, 3 from a
// scalar field)
// f3b (may be null) is subtracted from f3 node by node (the state change m_new - m_old)
__global__ void k_voxelise(const int* idx, const float* w, int nv, const double* f3, const double* f3b,
                           const double* f1, double s3, double s1, Vol v, uint4* x, int sample) {
  const int G = v.G;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    double acc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int nd = idx[4 * i + k];
      if (nd >= 0) {
        const double wk = w[4 * i + k];
        const size_t o = 3 * (size_t)nd;
        acc[0] += wk * (f3b ? f3[o] - f3b[o] : f3[o]);
        acc[1] += wk * (f3b ? f3[o + 1] - f3b[o + 1] : f3[o + 1]);
        acc[2] += wk * (f3b ? f3[o + 2] - f3b[o + 2] : f3[o + 2]);
        acc[3] += wk * f1[nd];
      }
    }
    const int xx = i % G, yy = (i / G) % G, z = i / (G * G);
    float f[8] = {(float)(acc[0] * s3), (float)(acc[1] * s3), (float)(acc[2] * s3), (float)(acc[3] * s1), 0, 0, 0, 0};
    x[(size_t)sample * 2 * v.plane + v.guard + flat(v, z, yy, xx)] = pack8(f);
  }
}

// grid -> mesh: U[node[j]] += scale * sum_k w[j][k] y0(voxel idx[j][k]) (8 voxels, trilinear)
__global__ void k_interp_add(const int* node, const int* idx, const float* w, int n, const uint4* y, Vol v, int nch,
                             int sample, double scale, double* U) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int vox = idx[8 * j + k];
      const int G = v.G;
      const int xx = vox % G, yy = (vox / G) % G, z = vox / (G * G);
      float f[8];
      unpack8(y[(size_t)sample * nch * v.plane + v.guard + flat(v, z, yy, xx)], f);
      acc += (double)w[8 * j + k] * (double)f[0];
    }
    U[node[j]] += scale * acc;
  }
}

}  // namespace mmn

// ================================================================================================
// host side
// ================================================================================================
namespace {

struct UFail {
  int code;
  std::string msg;
};

#define UCK(x)                                                                                        \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess)                                                                            \
      throw UFail{e_ == cudaErrorMemoryAllocation ? MM_ERR_OOM : MM_ERR_CUDA,                         \
                  std::string(#x) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +          \
                      std::to_string(__LINE__) + ")"};                                                \
  } while (0)

struct LayerDef {
  const char* name;
  int level, cin, cout;
  bool relu;
};
// the network (identical to the oracle's LAYERS)
const LayerDef DEFS[MM_UNET_LAYERS] = {
    {"e0a", 0, 16, 16, true},   {"e0b", 0, 16, 16, true},   {"e1a", 1, 16, 32, true},  {"e1b", 1, 32, 32, true},
    {"e2a", 2, 32, 64, true},   {"e2b", 2, 64, 64, true},   {"b3a", 3, 64, 128, true}, {"b3b", 3, 128, 128, true},
    {"b3c", 3, 128, 64, true},  {"d2a", 2, 64, 64, true},   {"d2b", 2, 64, 32, true},  {"d1a", 1, 32, 32, true},
    {"d1b", 1, 32, 16, true},   {"d0a", 0, 16, 16, true},   {"d0b", 0, 16, 16, false},
};
enum Lid { L_E0A, L_E0B, L_E1A, L_E1B, L_E2A, L_E2B, L_B3A, L_B3B, L_B3C, L_D2A, L_D2B, L_D1A, L_D1B, L_D0A, L_D0B };
// activation tensors (level, channels)
enum Tid { T_X, T_Y0A, T_S0, T_P0, T_Y1A, T_S1, T_P1, T_Y2A, T_S2, T_P2, T_Y3A, T_Y3B, T_Y3C, T_H2, T_YD2A, T_YD2B,
           T_H1, T_YD1A, T_YD1B, T_H0, T_YD0A, T_OUT, T_COUNT };
const int TDEF[T_COUNT][2] = {{0, 16}, {0, 16}, {0, 16}, {1, 16}, {1, 32}, {1, 32}, {2, 32}, {2, 64},
                              {2, 64}, {3, 64}, {3, 128}, {3, 128}, {3, 64}, {2, 64}, {2, 64}, {2, 32},
                              {1, 32}, {1, 32}, {1, 16}, {0, 16}, {0, 16}, {0, 16}};
constexpr int IN_CH = 4;
constexpr int NSPLIT_MAX = 64;

inline int nt_of(int cout) { return std::min(cout, 64); }
inline int cit_of(int cin) { return std::min(cin, 64); }

template <class F>
void conv_dispatch(int cin, int nt, F&& f) {
#define CONV_CASE(CI, NT_)                         \
  if (cin == CI && nt == NT_) {                    \
    f(mmn::k_conv_tc<CI, NT_>);                    \
    return;                                        \
  }
  CONV_CASE(16, 16) CONV_CASE(16, 32) CONV_CASE(16, 64) CONV_CASE(32, 16) CONV_CASE(32, 32) CONV_CASE(32, 64)
  CONV_CASE(64, 16) CONV_CASE(64, 32) CONV_CASE(64, 64) CONV_CASE(128, 16) CONV_CASE(128, 32) CONV_CASE(128, 64)
#undef CONV_CASE
  throw UFail{MM_ERR_ARG, "unsupported convolution shape"};
}

template <class F>
void wgrad_dispatch(int cit, int cot, F&& f) {
#define WG_CASE(A, B)                   \
  if (cit == A && cot == B) {           \
    f(mmn::k_wgrad<A, B>);              \
    return;                             \
  }
  WG_CASE(16, 16) WG_CASE(16, 32) WG_CASE(16, 64) WG_CASE(32, 16) WG_CASE(32, 32) WG_CASE(32, 64) WG_CASE(64, 16)
  WG_CASE(64, 32) WG_CASE(64, 64)
#undef WG_CASE
  throw UFail{MM_ERR_ARG, "unsupported weight-gradient shape"};
}

inline int grid1d(long long n, int bs = 256) { return (int)std::max<long long>(1, std::min<long long>((n + bs - 1) / bs, 8192)); }

}  // namespace

struct mm_unet {
  int G = 0, B = 0;
  cudaStream_t st = nullptr;
  std::string err;
  mmn::Vol vol[4];
  std::vector<void*> allocs;
  // parameters (flat FP32: per layer w[27][cin][cout] then b[cout]), gradients, Adam moments
  size_t nparam = 0;
  size_t woff[MM_UNET_LAYERS] = {}, boff[MM_UNET_LAYERS] = {};
  float *p = nullptr, *g = nullptr, *am = nullptr, *av = nullptr;
  int adam_t = 0;
  uint4* wk[MM_UNET_LAYERS] = {};
  uint4* wkT[MM_UNET_LAYERS] = {};
  // Layers whose forward grid would cover few CTAs (the coarse levels of a small grid) run with
  // 16-channel N tiles from a second weight copy: 4x the CTAs, each issuing a quarter of the MMA
  // work, the same accumulation order per output (identical results).
  uint4* wk16[MM_UNET_LAYERS] = {};
  uint4* T[T_COUNT] = {};
  uint4* dT[T_COUNT] = {};
  float* part = nullptr;
  size_t part_cap = 0;
  float* bpart = nullptr;
  double* lpart = nullptr;
  double* h_lpart = nullptr;
  float* stage_in = nullptr;   // FP32 [B][G^3][4]
  float* stage_t = nullptr;    // FP32 [B][G^3] (targets / outputs)
  int* d_err = nullptr;
  int nb_fwd = 0;              // samples of the last forward
  cudaGraphExec_t fwd_exec[8] = {};   // captured forward passes (batch sizes 1..8), on the in-place input
  bool fwd_warm = false;              // one forward has run (kernel attributes set) before any capture
  cudaEvent_t ev_after = nullptr;     // ordering point taken on a caller's stream (mm_unet_predict_dev)
  std::vector<std::pair<const void*, size_t>> attr_done;
  bool train_bias = true;      // false: bias gradients are zero (biases stay as set)

  template <class T>
  T* alloc(size_t n) {
    void* q = nullptr;
    UCK(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
    allocs.push_back(q);
    return (T*)q;
  }
  uint4* tensor(int level, int ch) {
    const size_t n = (size_t)B * (ch / 8) * vol[level].plane;
    uint4* q = alloc<uint4>(n);
    UCK(cudaMemsetAsync(q, 0, n * sizeof(uint4), st));
    return q;
  }
  // The network runs on its own non-blocking stream: an entry point that reads or writes a caller's
  // device arrays first orders that stream after the work queued so far on the legacy default stream
  // (where a caller such as torch queues the writes of those arrays).
  void after_caller() {
    if (!ev_after) UCK(cudaEventCreateWithFlags(&ev_after, cudaEventDisableTiming));
    UCK(cudaEventRecord(ev_after, cudaStreamLegacy));
    UCK(cudaStreamWaitEvent(st, ev_after, 0));
  }

  void check_err() {
    int e = 0;
    UCK(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    UCK(cudaStreamSynchronize(st));
    if (e) throw UFail{MM_ERR_CUDA, "a tensor-core convolution gave up waiting for its operands or accumulators"};
  }

  void conv(int l, const uint4* in, uint4* out, int nb, bool transposed) {
    const LayerDef& d = DEFS[l];
    const int cin = transposed ? d.cout : d.cin;
    const int cout = transposed ? d.cin : d.cout;
    const bool n16 = !transposed && wk16[l];
    const int nt = n16 ? 16 : nt_of(cout);
    const mmn::Vol& v = vol[d.level];
    mmn::ConvArgs a{};
    a.in = in;
    a.wk = transposed ? wkT[l] : (n16 ? wk16[l] : wk[l]);
    a.bias = transposed ? nullptr : p + boff[l];
    a.out = out;
    a.v = v;
    a.cin = cin;
    a.cout = cout;
    a.relu = (!transposed && d.relu) ? 1 : 0;
    a.err = d_err;
    const size_t smem = mmn::conv_smem(v.P, cin, nt);
    dim3 grid((unsigned)((v.t1 - v.t0 + 128 * mmn::MT - 1) / (128 * mmn::MT)), (unsigned)(cout / nt), (unsigned)nb);
    conv_dispatch(cin, nt, [&](auto kern) {
      // the kernel's shared-memory limit only ever grows (and is not touched during a graph capture
      // once every size has been seen)
      size_t* cur = nullptr;
      for (auto& kv : attr_done)
        if (kv.first == (const void*)kern) cur = &kv.second;
      if (!cur) {
        attr_done.emplace_back((const void*)kern, 0);
        cur = &attr_done.back().second;
      }
      if (smem > *cur) {
        UCK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        *cur = smem;
      }
      kern<<<grid, 128, smem, st>>>(a);
      UCK(cudaGetLastError());
    });
  }

  // voxels per block and splits of the weight-gradient reduction of a layer
  void wg_split(int l, int nb, int& vpb, int& ns) const {
    const LayerDef& d = DEFS[l];
    const mmn::Vol& v = vol[d.level];
    const int range = v.t1 - v.t0;
    const int tiles = 27 * (d.cin / cit_of(d.cin)) * (d.cout / nt_of(d.cout));
    ns = std::max(1, std::min(NSPLIT_MAX, 2048 / std::max(1, tiles * nb)));
    ns = std::min(ns, (range + 63) / 64);
    vpb = ((range + ns - 1) / ns + 63) / 64 * 64;
    ns = (range + vpb - 1) / vpb;
  }

  void bwd_layer(int l, uint4* dy, const uint4* x, const uint4* y, uint4* dx, int nb) {
    const LayerDef& d = DEFS[l];
    const mmn::Vol& v = vol[d.level];
    if (d.relu) {
      const long long n = (long long)nb * (d.cout / 8) * v.G * v.G * v.G;
      mmn::k_relu_mask<<<grid1d(n), 256, 0, st>>>(dy, y, v, d.cout / 8, nb);
      UCK(cudaGetLastError());
    }
    int vpb = 0, ns = 0;
    wg_split(l, nb, vpb, ns);
    mmn::WgArgs a{};
    a.x = x;
    a.d = dy;
    a.part = part;
    a.v = v;
    a.cin = d.cin;
    a.cout = d.cout;
    a.vpb = vpb;
    a.nsplit = ns;
    const int cit = cit_of(d.cin), cot = nt_of(d.cout);
    dim3 grid((unsigned)ns, (unsigned)(27 * (d.cin / cit) * (d.cout / cot)), (unsigned)nb);
    wgrad_dispatch(cit, cot, [&](auto kern) {
      kern<<<grid, 128, 0, st>>>(a);
      UCK(cudaGetLastError());
    });
    const int nw = 27 * d.cin * d.cout;
    mmn::k_sum_parts<<<grid1d(nw), 256, 0, st>>>(part, nb * ns, nw, d.cin, d.cout, l == L_E0A ? IN_CH : d.cin,
                                                 g + woff[l]);
    UCK(cudaGetLastError());
    if (train_bias) {
      mmn::k_bias_part<<<dim3((unsigned)ns, (unsigned)nb), 128, 0, st>>>(dy, v, d.cout, vpb, ns, bpart);
      UCK(cudaGetLastError());
      mmn::k_sum_parts<<<grid1d(d.cout), 256, 0, st>>>(bpart, nb * ns, d.cout, 1, d.cout, 1, g + boff[l]);
      UCK(cudaGetLastError());
    } else {
      UCK(cudaMemsetAsync(g + boff[l], 0, d.cout * sizeof(float), st));
    }
    if (dx) conv(l, dy, dx, nb, true);
  }

  void prep_weights() {
    for (int l = 0; l < MM_UNET_LAYERS; ++l) {
      const LayerDef& d = DEFS[l];
      const int nf = (d.cout / nt_of(d.cout)) * (d.cin / 16) * 54 * nt_of(d.cout);
      mmn::k_prep_weights<<<grid1d(nf), 256, 0, st>>>(p + woff[l], d.cin, d.cout, nt_of(d.cout), 0, wk[l]);
      UCK(cudaGetLastError());
      const int nt2 = (d.cin / nt_of(d.cin)) * (d.cout / 16) * 54 * nt_of(d.cin);
      mmn::k_prep_weights<<<grid1d(nt2), 256, 0, st>>>(p + woff[l], d.cin, d.cout, nt_of(d.cin), 1, wkT[l]);
      UCK(cudaGetLastError());
      if (wk16[l]) {
        mmn::k_prep_weights<<<grid1d(nf), 256, 0, st>>>(p + woff[l], d.cin, d.cout, 16, 0, wk16[l]);
        UCK(cudaGetLastError());
      }
    }
  }

  void pool(int tf, int tc, int nb) {
    const mmn::Vol &vf = vol[TDEF[tf][0]], &vc = vol[TDEF[tc][0]];
    const int nch = TDEF[tf][1] / 8;
    mmn::k_pool<<<grid1d((long long)nb * nch * vc.G * vc.G * vc.G), 256, 0, st>>>(T[tf], vf, T[tc], vc, nch, nb);
    UCK(cudaGetLastError());
  }
  void up_add(int tc, int tskip, int tout, int nb) {
    const mmn::Vol &vc = vol[TDEF[tc][0]], &vf = vol[TDEF[tout][0]];
    const int nch = TDEF[tout][1] / 8;
    mmn::k_up_add<<<grid1d((long long)nb * nch * vf.G * vf.G * vf.G), 256, 0, st>>>(T[tc], vc, T[tskip], T[tout], vf,
                                                                                   nch, nb);
    UCK(cudaGetLastError());
  }
  void up_bwd(int tf, int tc, int nb) {  // dT[tc] = sum of children of dT[tf]
    const mmn::Vol &vf = vol[TDEF[tf][0]], &vc = vol[TDEF[tc][0]];
    const int nch = TDEF[tc][1] / 8;
    mmn::k_up_bwd<<<grid1d((long long)nb * nch * vc.G * vc.G * vc.G), 256, 0, st>>>(dT[tf], vf, dT[tc], vc, nch, nb);
    UCK(cudaGetLastError());
  }
  void pool_bwd_add(int tc, int tskip, int tf, int nb) {  // dT[tf] = dT[tc]/8 + dT[tskip]
    const mmn::Vol &vc = vol[TDEF[tc][0]], &vf = vol[TDEF[tf][0]];
    const int nch = TDEF[tf][1] / 8;
    mmn::k_pool_bwd_add<<<grid1d((long long)nb * nch * vf.G * vf.G * vf.G), 256, 0, st>>>(dT[tc], vc, dT[tskip],
                                                                                         dT[tf], vf, nch, nb);
    UCK(cudaGetLastError());
  }

  // forward on T[T_X] (already packed)
  void forward(int nb) {
    conv(L_E0A, T[T_X], T[T_Y0A], nb, false);
    conv(L_E0B, T[T_Y0A], T[T_S0], nb, false);
    pool(T_S0, T_P0, nb);
    conv(L_E1A, T[T_P0], T[T_Y1A], nb, false);
    conv(L_E1B, T[T_Y1A], T[T_S1], nb, false);
    pool(T_S1, T_P1, nb);
    conv(L_E2A, T[T_P1], T[T_Y2A], nb, false);
    conv(L_E2B, T[T_Y2A], T[T_S2], nb, false);
    pool(T_S2, T_P2, nb);
    conv(L_B3A, T[T_P2], T[T_Y3A], nb, false);
    conv(L_B3B, T[T_Y3A], T[T_Y3B], nb, false);
    conv(L_B3C, T[T_Y3B], T[T_Y3C], nb, false);
    up_add(T_Y3C, T_S2, T_H2, nb);
    conv(L_D2A, T[T_H2], T[T_YD2A], nb, false);
    conv(L_D2B, T[T_YD2A], T[T_YD2B], nb, false);
    up_add(T_YD2B, T_S1, T_H1, nb);
    conv(L_D1A, T[T_H1], T[T_YD1A], nb, false);
    conv(L_D1B, T[T_YD1A], T[T_YD1B], nb, false);
    up_add(T_YD1B, T_S0, T_H0, nb);
    conv(L_D0A, T[T_H0], T[T_YD0A], nb, false);
    conv(L_D0B, T[T_YD0A], T[T_OUT], nb, false);
    nb_fwd = nb;
  }

  // loss against FP32 targets on the device; gradients of every parameter into g
  double backward(const float* d_target, int nb) {
    const mmn::Vol& v0 = vol[0];
    mmn::k_loss<<<256, 256, 0, st>>>(T[T_OUT], v0, 2, d_target, nb, dT[T_OUT], lpart);
    UCK(cudaGetLastError());
    UCK(cudaMemcpyAsync(h_lpart, lpart, 256 * sizeof(double), cudaMemcpyDeviceToHost, st));
    bwd_layer(L_D0B, dT[T_OUT], T[T_YD0A], T[T_OUT], dT[T_YD0A], nb);
    bwd_layer(L_D0A, dT[T_YD0A], T[T_H0], T[T_YD0A], dT[T_H0], nb);
    up_bwd(T_H0, T_YD1B, nb);
    bwd_layer(L_D1B, dT[T_YD1B], T[T_YD1A], T[T_YD1B], dT[T_YD1A], nb);
    bwd_layer(L_D1A, dT[T_YD1A], T[T_H1], T[T_YD1A], dT[T_H1], nb);
    up_bwd(T_H1, T_YD2B, nb);
    bwd_layer(L_D2B, dT[T_YD2B], T[T_YD2A], T[T_YD2B], dT[T_YD2A], nb);
    bwd_layer(L_D2A, dT[T_YD2A], T[T_H2], T[T_YD2A], dT[T_H2], nb);
    up_bwd(T_H2, T_Y3C, nb);
    bwd_layer(L_B3C, dT[T_Y3C], T[T_Y3B], T[T_Y3C], dT[T_Y3B], nb);
    bwd_layer(L_B3B, dT[T_Y3B], T[T_Y3A], T[T_Y3B], dT[T_Y3A], nb);
    bwd_layer(L_B3A, dT[T_Y3A], T[T_P2], T[T_Y3A], dT[T_P2], nb);
    pool_bwd_add(T_P2, T_H2, T_S2, nb);
    bwd_layer(L_E2B, dT[T_S2], T[T_Y2A], T[T_S2], dT[T_Y2A], nb);
    bwd_layer(L_E2A, dT[T_Y2A], T[T_P1], T[T_Y2A], dT[T_P1], nb);
    pool_bwd_add(T_P1, T_H1, T_S1, nb);
    bwd_layer(L_E1B, dT[T_S1], T[T_Y1A], T[T_S1], dT[T_Y1A], nb);
    bwd_layer(L_E1A, dT[T_Y1A], T[T_P0], T[T_Y1A], dT[T_P0], nb);
    pool_bwd_add(T_P0, T_H0, T_S0, nb);
    bwd_layer(L_E0B, dT[T_S0], T[T_Y0A], T[T_S0], dT[T_Y0A], nb);
    bwd_layer(L_E0A, dT[T_Y0A], T[T_X], T[T_Y0A], nullptr, nb);
    check_err();
    double s = 0.0;
    for (int i = 0; i < 256; ++i) s += h_lpart[i];
    return s / ((double)nb * v0.G * v0.G * v0.G);
  }

  void adam(float lr, float b1, float b2, float eps) {
    ++adam_t;
    const float c1 = 1.0f - std::pow(b1, (float)adam_t), c2 = 1.0f - std::pow(b2, (float)adam_t);
    mmn::k_adam<<<grid1d((long long)nparam), 256, 0, st>>>(p, g, am, av, nparam, lr, b1, b2, eps, c1, c2);
    UCK(cudaGetLastError());
    prep_weights();
  }
};

namespace {
thread_local std::string g_unet_error;

template <class F>
int uguard(mm_unet* u, F&& f) {
  try {
    return f();
  } catch (const UFail& e) {
    if (u) u->err = e.msg;
    else g_unet_error = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    if (u) u->err = e.what();
    else g_unet_error = e.what();
    return MM_ERR_SETUP;
  }
}
}  // namespace

extern "C" {

int mm_unet_create(int grid, int batch, mm_unet** out) {
  if (!out || grid < 16 || grid % 8 != 0 || grid > 256 || batch < 1) return MM_ERR_ARG;
  *out = nullptr;
  mm_unet* u = new mm_unet();
  const int rc = uguard(u, [&] {
    u->G = grid;
    u->B = batch;
    UCK(cudaStreamCreateWithFlags(&u->st, cudaStreamNonBlocking));
    for (int l = 0; l < 4; ++l) u->vol[l] = mmn::make_vol(grid >> l);
    size_t off = 0;
    for (int l = 0; l < MM_UNET_LAYERS; ++l) {
      u->woff[l] = off;
      off += (size_t)27 * DEFS[l].cin * DEFS[l].cout;
      u->boff[l] = off;
      off += DEFS[l].cout;
    }
    u->nparam = off;
    u->p = u->alloc<float>(off);
    u->g = u->alloc<float>(off);
    u->am = u->alloc<float>(off);
    u->av = u->alloc<float>(off);
    UCK(cudaMemsetAsync(u->p, 0, off * sizeof(float), u->st));
    UCK(cudaMemsetAsync(u->g, 0, off * sizeof(float), u->st));
    UCK(cudaMemsetAsync(u->am, 0, off * sizeof(float), u->st));
    UCK(cudaMemsetAsync(u->av, 0, off * sizeof(float), u->st));
    for (int l = 0; l < MM_UNET_LAYERS; ++l) {
      u->wk[l] = u->alloc<uint4>((size_t)27 * 2 * DEFS[l].cin / 16 * DEFS[l].cout);
      u->wkT[l] = u->alloc<uint4>((size_t)27 * 2 * DEFS[l].cout / 16 * DEFS[l].cin);
      // fewer than half an SM's worth of CTAs per sample with the default N tile: also keep N = 16
      const mmn::Vol& v = u->vol[DEFS[l].level];
      const int tiles = (v.t1 - v.t0 + 128 * mmn::MT - 1) / (128 * mmn::MT);
      if (DEFS[l].cout > 16 && tiles * (DEFS[l].cout / nt_of(DEFS[l].cout)) < 76)
        u->wk16[l] = u->alloc<uint4>((size_t)27 * 2 * DEFS[l].cin / 16 * DEFS[l].cout);
    }
    for (int t = 0; t < T_COUNT; ++t) {
      u->T[t] = u->tensor(TDEF[t][0], TDEF[t][1]);
      u->dT[t] = u->tensor(TDEF[t][0], TDEF[t][1]);
    }
    size_t cap = 0, bcap = 0;
    for (int l = 0; l < MM_UNET_LAYERS; ++l) {
      int vpb = 0, ns = 0;
      u->wg_split(l, batch, vpb, ns);
      cap = std::max(cap, (size_t)batch * ns * 27 * DEFS[l].cin * DEFS[l].cout);
      bcap = std::max(bcap, (size_t)batch * ns * DEFS[l].cout);
      for (int nb = 1; nb < batch; ++nb) {  // smaller batches split further
        u->wg_split(l, nb, vpb, ns);
        cap = std::max(cap, (size_t)nb * ns * 27 * DEFS[l].cin * DEFS[l].cout);
        bcap = std::max(bcap, (size_t)nb * ns * DEFS[l].cout);
      }
    }
    u->part = u->alloc<float>(cap);
    u->part_cap = cap;
    u->bpart = u->alloc<float>(bcap);
    u->lpart = u->alloc<double>(256);
    UCK(cudaMallocHost(&u->h_lpart, 256 * sizeof(double)));
    const size_t nv = (size_t)batch * grid * grid * grid;
    u->stage_in = u->alloc<float>(nv * 4);
    u->stage_t = u->alloc<float>(nv);
    u->d_err = u->alloc<int>(1);
    UCK(cudaMemsetAsync(u->d_err, 0, sizeof(int), u->st));
    UCK(cudaStreamSynchronize(u->st));
    return MM_OK;
  });
  if (rc != MM_OK) {
    g_unet_error = u->err;
    for (void* q : u->allocs) cudaFree(q);
    if (u->h_lpart) cudaFreeHost(u->h_lpart);
    if (u->st) cudaStreamDestroy(u->st);
    delete u;
    return rc;
  }
  *out = u;
  return MM_OK;
}

int mm_unet_destroy(mm_unet* u) {
  if (!u) return MM_ERR_ARG;
  if (u->st) cudaStreamSynchronize(u->st);
  for (cudaGraphExec_t e : u->fwd_exec)
    if (e) cudaGraphExecDestroy(e);
  for (void* q : u->allocs) cudaFree(q);
  if (u->h_lpart) cudaFreeHost(u->h_lpart);
  if (u->ev_after) cudaEventDestroy(u->ev_after);
  if (u->st) cudaStreamDestroy(u->st);
  delete u;
  return MM_OK;
}

const char* mm_unet_last_error(mm_unet* u) { return u ? u->err.c_str() : g_unet_error.c_str(); }

int mm_unet_param_count(mm_unet* u, int64_t* n) {
  if (!u || !n) return MM_ERR_ARG;
  *n = (int64_t)u->nparam;
  return MM_OK;
}

int mm_unet_set_params(mm_unet* u, const float* params) {
  if (!u || !params) return MM_ERR_ARG;
  return uguard(u, [&] {
    UCK(cudaMemcpyAsync(u->p, params, u->nparam * sizeof(float), cudaMemcpyHostToDevice, u->st));
    UCK(cudaMemsetAsync(u->am, 0, u->nparam * sizeof(float), u->st));
    UCK(cudaMemsetAsync(u->av, 0, u->nparam * sizeof(float), u->st));
    u->adam_t = 0;
    u->prep_weights();
    UCK(cudaStreamSynchronize(u->st));
    return MM_OK;
  });
}

int mm_unet_get_params(mm_unet* u, float* params) {
  if (!u || !params) return MM_ERR_ARG;
  return uguard(u, [&] {
    UCK(cudaMemcpyAsync(params, u->p, u->nparam * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    UCK(cudaStreamSynchronize(u->st));
    return MM_OK;
  });
}

int mm_unet_get_grads(mm_unet* u, float* grads) {
  if (!u || !grads) return MM_ERR_ARG;
  return uguard(u, [&] {
    UCK(cudaMemcpyAsync(grads, u->g, u->nparam * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    UCK(cudaStreamSynchronize(u->st));
    return MM_OK;
  });
}

int mm_unet_forward(mm_unet* u, const float* x, int nb, float* y) {
  if (!u || !x || nb < 1 || nb > u->B) return MM_ERR_ARG;
  return uguard(u, [&] {
    const size_t nv = (size_t)nb * u->G * u->G * u->G;
    UCK(cudaMemcpyAsync(u->stage_in, x, nv * 4 * sizeof(float), cudaMemcpyHostToDevice, u->st));
    mmn::k_pack_input<<<grid1d((long long)nv), 256, 0, u->st>>>(u->stage_in, u->vol[0], u->T[T_X], nb);
    UCK(cudaGetLastError());
    u->forward(nb);
    if (y) {
      mmn::k_unpack_out<<<grid1d((long long)nv), 256, 0, u->st>>>(u->T[T_OUT], u->vol[0], 2, u->stage_t, nb);
      UCK(cudaGetLastError());
      UCK(cudaMemcpyAsync(y, u->stage_t, nv * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    }
    u->check_err();
    return MM_OK;
  });
}

// The forward on the in-place input as one CUDA graph (captured at the second call for each batch
// size), without a wait; errors are reported by the next call that waits.
static void forward_graph(mm_unet* u, int nb) {
  if (!u->fwd_warm) {
    u->forward(nb);
    u->check_err();
    u->fwd_warm = true;
    return;
  }
  if (!u->fwd_exec[nb - 1]) {
    cudaGraph_t g = nullptr;
    UCK(cudaStreamBeginCapture(u->st, cudaStreamCaptureModeThreadLocal));
    u->forward(nb);
    UCK(cudaStreamEndCapture(u->st, &g));
    UCK(cudaGraphInstantiate(&u->fwd_exec[nb - 1], g, 0));
    cudaGraphDestroy(g);
  }
  UCK(cudaGraphLaunch(u->fwd_exec[nb - 1], u->st));
  u->nb_fwd = nb;
}

int mm_unet_forward_dev(mm_unet* u, const float* d_x, int nb, float* d_y) {
  if (!u || nb < 1 || nb > u->B) return MM_ERR_ARG;
  return uguard(u, [&] {
    const size_t nv = (size_t)nb * u->G * u->G * u->G;
    if (!d_x && !d_y && nb <= 8) {
      // in-place input, output left in the network (errors: mm_unet_interp_add_dev or mm_unet_sync)
      forward_graph(u, nb);
      return MM_OK;
    }
    u->after_caller();
    if (d_x) {
      mmn::k_pack_input<<<grid1d((long long)nv), 256, 0, u->st>>>(d_x, u->vol[0], u->T[T_X], nb);
      UCK(cudaGetLastError());
    }
    u->forward(nb);
    if (d_y) {
      mmn::k_unpack_out<<<grid1d((long long)nv), 256, 0, u->st>>>(u->T[T_OUT], u->vol[0], 2, d_y, nb);
      UCK(cudaGetLastError());
    }
    u->check_err();
    return MM_OK;
  });
}

int mm_unet_backward(mm_unet* u, const float* target, int nb, double* loss) {
  if (!u || !target || nb < 1 || nb != u->nb_fwd) return MM_ERR_ARG;
  return uguard(u, [&] {
    const size_t nv = (size_t)nb * u->G * u->G * u->G;
    UCK(cudaMemcpyAsync(u->stage_t, target, nv * sizeof(float), cudaMemcpyHostToDevice, u->st));
    const double L = u->backward(u->stage_t, nb);
    if (loss) *loss = L;
    return MM_OK;
  });
}

int mm_unet_backward_dev(mm_unet* u, const float* d_target, int nb, double* loss) {
  if (!u || !d_target || nb < 1 || nb != u->nb_fwd) return MM_ERR_ARG;
  return uguard(u, [&] {
    u->after_caller();
    const double L = u->backward(d_target, nb);
    if (loss) *loss = L;
    return MM_OK;
  });
}

int mm_unet_set_bias_training(mm_unet* u, int on) {
  if (!u || (on != 0 && on != 1)) return MM_ERR_ARG;
  u->train_bias = on == 1;
  return MM_OK;
}

int mm_unet_adam(mm_unet* u, float lr, float beta1, float beta2, float eps) {
  if (!u || !(lr > 0)) return MM_ERR_ARG;
  return uguard(u, [&] {
    u->adam(lr, beta1, beta2, eps);
    return MM_OK;
  });
}

int mm_unet_voxelise_dev(mm_unet* u, int sample, int n_vox, const int* d_idx4, const float* d_w4, const double* d_f3,
                         const double* d_f1, double scale3, double scale1) {
  if (!u || sample < 0 || sample >= u->B || n_vox != u->G * u->G * u->G || !d_idx4 || !d_w4 || !d_f3 || !d_f1)
    return MM_ERR_ARG;
  return uguard(u, [&] {
    u->after_caller();
    mmn::k_voxelise<<<grid1d(n_vox), 256, 0, u->st>>>(d_idx4, d_w4, n_vox, d_f3, nullptr, d_f1, scale3, scale1,
                                                       u->vol[0], u->T[T_X], sample);
    UCK(cudaGetLastError());
    return MM_OK;
  });
}

int mm_unet_interp_add_dev(mm_unet* u, int sample, int n, const int* d_node, const int* d_idx8, const float* d_w8,
                           double scale, double* d_U) {
  if (!u || sample < 0 || sample >= u->B || n < 0 || (n > 0 && (!d_node || !d_idx8 || !d_w8 || !d_U)))
    return MM_ERR_ARG;
  return uguard(u, [&] {
    if (n > 0) {
      u->after_caller();
      mmn::k_interp_add<<<grid1d(n), 256, 0, u->st>>>(d_node, d_idx8, d_w8, n, u->T[T_OUT], u->vol[0], 2, sample,
                                                        scale, d_U);
      UCK(cudaGetLastError());
    }
    u->check_err();
    return MM_OK;
  });
}

int mm_unet_tensor_info(int which, int* level, int* channels) {
  if (which < 0 || which >= T_COUNT || !level || !channels) return MM_ERR_ARG;
  *level = TDEF[which][0];
  *channels = TDEF[which][1];
  return MM_OK;
}

int mm_unet_read_tensor(mm_unet* u, int which, int grad, int sample, float* out) {
  if (!u || which < 0 || which >= T_COUNT || sample < 0 || sample >= u->B || !out) return MM_ERR_ARG;
  return uguard(u, [&] {
    const mmn::Vol& v = u->vol[TDEF[which][0]];
    const int nch = TDEF[which][1] / 8;
    const size_t n = (size_t)v.G * v.G * v.G * nch * 8;
    float* d = u->alloc<float>(n);
    mmn::k_read_tensor<<<grid1d((long long)n / 8), 256, 0, u->st>>>(grad ? u->dT[which] : u->T[which], v, nch,
                                                                     sample, d);
    UCK(cudaGetLastError());
    UCK(cudaMemcpyAsync(out, d, n * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    UCK(cudaStreamSynchronize(u->st));
    UCK(cudaFree(d));
    u->allocs.pop_back();
    return MM_OK;
  });
}

int mm_unet_predict_dev(mm_unet* u, void* after, int sample, int n_vox, const int* d_idx4, const float* d_w4,
                        const double* d_f3a, const double* d_f3b, const double* d_f1, double scale3, double scale1,
                        int n, const int* d_node, const int* d_idx8, const float* d_w8, double scale, int n_out,
                        double* d_out, void** stream_out) {
  if (!u || sample != 0 || n_vox != u->G * u->G * u->G || !d_idx4 || !d_w4 || !d_f3a || !d_f1 || n < 0 ||
      n_out < 0 || (n > 0 && (!d_node || !d_idx8 || !d_w8)) || (n_out > 0 && !d_out))
    return MM_ERR_ARG;
  return uguard(u, [&] {
    if (!u->ev_after) UCK(cudaEventCreateWithFlags(&u->ev_after, cudaEventDisableTiming));
    UCK(cudaEventRecord(u->ev_after, (cudaStream_t)after));
    UCK(cudaStreamWaitEvent(u->st, u->ev_after, 0));
    mmn::k_voxelise<<<grid1d(n_vox), 256, 0, u->st>>>(d_idx4, d_w4, n_vox, d_f3a, d_f3b, d_f1, scale3, scale1,
                                                       u->vol[0], u->T[T_X], 0);
    UCK(cudaGetLastError());
    forward_graph(u, 1);
    if (n_out > 0) UCK(cudaMemsetAsync(d_out, 0, (size_t)n_out * sizeof(double), u->st));
    if (n > 0) {
      mmn::k_interp_add<<<grid1d(n), 256, 0, u->st>>>(d_node, d_idx8, d_w8, n, u->T[T_OUT], u->vol[0], 2, 0, scale,
                                                        d_out);
      UCK(cudaGetLastError());
    }
    if (stream_out) *stream_out = (void*)u->st;
    return MM_OK;
  });
}

int mm_unet_sync(mm_unet* u) {
  if (!u) return MM_ERR_ARG;
  return uguard(u, [&] {
    u->check_err();
    return MM_OK;
  });
}

}  // extern "C"
