// pfchem_mlp.cu -- learned warm start for the per-cell Newton solve.
//
// A 16 -> 256 -> 256 -> 256 -> 12 multilayer perceptron (GELU) maps per-cell
// features of the step -- the signed-log totals that the step conserves
// (aqueous plus sorbed, per litre of pore water), a pH proxy, temperature and
// the ionic strength of the previous state -- to the 12 log-molalities of the
// step's solution.  Weights and activations are BF16, products accumulate in
// FP32 on the tensor cores (mma.sync m16n8k16), and it is trained here, with
// these kernels, on solves produced by the FP64 Newton kernel itself.  FP64
// Newton always finishes every cell: the prediction enters as the solve's
// alternative guess, taken per cell only if its first residual is no worse
// than the previous-step guess's.
//
// Kernels: one tiled BF16 GEMM (operands read through arbitrary row/column
// strides, so the same kernel serves X W, dY W^T and X^T dY) with fused
// bias + GELU epilogues; GELU backward; bias gradients; the MSE loss and its
// gradient; AdamW on FP32 master weights (refreshing the BF16 copies); the
// feature and output transforms.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "pfchem_device.cuh"

namespace pfchem {

cudaError_t umma_prepare();
bool umma_supports(int N, int K, bool w_kn);
cudaError_t umma_linear(cudaStream_t st, const __nv_bfloat16 *X, long long rows, int K, const __nv_bfloat16 *W, int N,
                        bool w_kn, const float *bias, float *Cf, __nv_bfloat16 *Cb, int epi, int *err, int sms,
                        __nv_bfloat16 *bpk);
constexpr int kUmmaGeluE = 0, kUmmaLinearE = 1;  // umma_linear epilogues

constexpr int kFeat = 16;    // input features
constexpr int kHidden = 256;  // hidden width
constexpr int kOut = PFCHEM_MAX_PRI;  // outputs (the first N used)
constexpr int kLayers = 4;

namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C(m, n) = sum_k A(m, k) B(k, n), A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn].
// Epilogues: kEpiAct: Cf = acc + bias (FP32), Cb = act(acc + bias) (BF16);
//            kEpiF32: Cf = acc (+ bias); kEpiAccF32: Cf += acc (FP32 accumulate, no bias).
enum { kEpiAct = 0, kEpiF32 = 1 };
constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// One BR x BK tile of a strided BF16 operand X(r, k) = X[r*sr + k*sk] into
// T[r][k] (k contiguous in shared memory).  When one stride is 1 the global
// loads are 16-byte vectors along it (8 elements): along k they land in one
// shared-memory row, along r they are scattered down a column.  Out-of-range
// elements are zero.
template <int BR>
__device__ __forceinline__ void load_tile(bf16 (*T)[BK + PAD], const bf16 *__restrict__ X, long long sr, long long sk,
                                          int R, int K, int r0, int k0, int tid) {
  const bf16 zero = __float2bfloat16(0.f);
  if (sk == 1) {
    for (int e = tid; e < BR * BK / 8; e += 128) {
      const int rr = e / (BK / 8), kk = (e % (BK / 8)) * 8;
      const int gr = r0 + rr, gk = k0 + kk;
      const bf16 *src = X + (long long)gr * sr + gk;
      if (gr < R && gk + 8 <= K && aligned16(src)) {
        *reinterpret_cast<uint4 *>(&T[rr][kk]) = *reinterpret_cast<const uint4 *>(src);
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) T[rr][kk + q] = (gr < R && gk + q < K) ? src[q] : zero;
      }
    }
  } else if (sr == 1) {
    for (int e = tid; e < BR * BK / 8; e += 128) {
      const int kk = e / (BR / 8), rr = (e % (BR / 8)) * 8;
      const int gr = r0 + rr, gk = k0 + kk;
      const bf16 *src = X + (long long)gk * sk + gr;
      if (gk < K && gr + 8 <= R && aligned16(src)) {
        uint4 v = *reinterpret_cast<const uint4 *>(src);
        const bf16 *h = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
        for (int q = 0; q < 8; ++q) T[rr + q][kk] = h[q];
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) T[rr + q][kk] = (gk < K && gr + q < R) ? src[q] : zero;
      }
    }
  } else {
    for (int e = tid; e < BR * BK; e += 128) {
      const int rr = e / BK, kk = e % BK;
      const int gr = r0 + rr, gk = k0 + kk;
      T[rr][kk] = (gr < R && gk < K) ? X[(long long)gr * sr + (long long)gk * sk] : zero;
    }
  }
}

// C(m, n) = sum_k A(m, k) B(k, n), A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn].
// Epilogues: kEpiAct: Cf = acc + bias (FP32), Cb = act(acc + bias) (BF16);
//            kEpiF32: Cf = acc (+ bias).
// Split K: block z sums k in [z*kchunk, (z+1)*kchunk) and, with more than
// one split, writes its partial product to Cf + z*M*ldc (no bias); the
// partials are then summed in a fixed order by sum_splits.
template <int EPI>
__global__ void __launch_bounds__(128) gemm_bf16(const bf16 *__restrict__ A, long long sam, long long sak,
                                                  const bf16 *__restrict__ B, long long sbk, long long sbn, int M,
                                                  int N, int K, const float *__restrict__ bias, float *Cf, bf16 *Cb,
                                                  int ldc, int act, int kchunk) {
  __shared__ __align__(16) bf16 As[BM][BK + PAD];
  __shared__ __align__(16) bf16 Bs[BN][BK + PAD];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  for (int k0 = kb; k0 < ke; k0 += BK) {
    load_tile<BM>(As, A, sam, sak, M, ke, m0, k0, tid);
    load_tile<BN>(Bs, B, sbn, sbk, N, ke, n0, k0, tid);
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm * 32 + i * 16 + g;
        a[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * t]);
        a[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * t]);
        a[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * t + 8]);
        a[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn * 32 + j * 8 + g;
        b[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * t]);
        b[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma16816(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const bool split = gridDim.z > 1;
  float *Co = split ? Cf + (long long)blockIdx.z * M * ldc : Cf;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = m0 + wm * 32 + i * 16 + g + (q >= 2 ? 8 : 0);
        const int c = n0 + wn * 32 + j * 8 + 2 * t + (q & 1);
        if (r < M && c < N) {
          float z = acc[i][j][q] + ((bias && !split) ? bias[c] : 0.f);
          const long long o = (long long)r * ldc + c;
          if (EPI == kEpiAct) {
            if (Cf) Cf[o] = z;
            Cb[o] = __float2bfloat16(act ? gelu(z) : z);
          } else {
            Co[o] = z;
          }
        }
      }
}

// out[i] = sum over the splits of part[z][i], in split order
__global__ void sum_splits(const float *__restrict__ part, float *out, long long n, int splits) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(long long)z * n + i];
  out[i] = s;
}

// dZ = dH * GELU'(Z), dH given in FP32; output BF16 (GEMM operand) and FP32 kept
__global__ void gelu_backward(const float *__restrict__ dH, const float *__restrict__ Z, bf16 *dZb, float *dZf,
                              long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = dH[i] * gelu_grad(Z[i]);
  dZb[i] = __float2bfloat16(v);
  if (dZf) dZf[i] = v;
}

// db[c] = sum_r dZ[r, c] (rows split over blockIdx.y, atomics into db)
__global__ void bias_grad(const float *__restrict__ dZ, float *db, int M, int N) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int rows_per = (M + gridDim.y - 1) / gridDim.y;
  const int r0 = blockIdx.y * rows_per, r1 = min(M, r0 + rows_per);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += dZ[(long long)r * N + c];
  atomicAdd(&db[c], s);
}

// MSE over the first `nout` outputs: dY = 2 (Y - T) / (M nout), loss sum
__global__ void mse_loss(const float *__restrict__ Y, const float *__restrict__ T, float *dY, bf16 *dYb, int M,
                         int ldy, int nout, float *loss) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < (long long)M * ldy) {
    const int c = (int)(i % ldy);
    float d = 0.f;
    if (c < nout) {
      const long long r = i / ldy;
      d = Y[i] - T[r * nout + c];
      l = d * d;
    }
    const float gval = 2.f * d / ((float)M * nout);
    dY[i] = gval;
    dYb[i] = __float2bfloat16(gval);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

__global__ void adamw(float *w, bf16 *wb, const float *g, float *m, float *v, long long n, float lr, float b1,
                      float b2, float eps, float wd, float bc1, float bc2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float wi = w[i] * (1.f - lr * wd);
  wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void to_bf16(const float *x, bf16 *y, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// Per-cell features (raw, before standardisation) of one cell into x[kFeat].
// The conserved totals are formed in FP64; the logarithms are taken in FP32,
// which is far finer than the BF16 the network reads them in (and keeps the
// FP64 pipe for the Newton work).
// One out-of-line copy serves both inference paths: inlined, the FP32 math
// functions can be contracted differently in each kernel.
__device__ __noinline__ void features_of(const CellArgs &a, int N, int sorb, long long cell, float *x) {
  const long long nc = a.ncells;
  const double por = a.por[cell], sat = a.sat[cell], vol = a.vol[cell];
  const double psv = __dmul_rn(__dmul_rn(__dmul_rn(por, sat), 1000.0), vol);
  const double ipsv = __ddiv_rn(1e12, psv);
  for (int j = 0; j < kFeat; ++j) x[j] = 0.f;
  // explicitly rounded operations: the value must not depend on where the
  // compiler contracts to FMA (the fused and the layer-by-layer paths inline
  // this function in different kernels)
  for (int j = 0; j < N; ++j) {
    double acc = __dmul_rn(psv, a.total[j * a.total_stride_comp + cell * a.total_stride_cell]);
    if (sorb) acc = __fma_rn(vol, a.sorb[j * nc + cell], acc);
    x[j] = asinhf(__double2float_rn(__dmul_rn(acc, ipsv)));  // signed log of the conserved total [mol/L]
  }
  x[12] = -log10f(fmaxf((float)a.pri_molal[cell], 1e-37f));  // pH proxy: the H+-like first species of the guess
  x[13] = (float)a.temp[cell];
  x[14] = log10f(fmaxf((float)a.ionic[cell], 1e-30f));
}

// Per-cell features, row-major [cell][kFeat].
__global__ void cell_features(const CellArgs a, int N, int sorb, float *X) {
  const long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (cell >= a.ncells) return;
  features_of(a, N, sorb, cell, X + cell * kFeat);
}

// ---------------------------------------------------------------------------
// Fused inference: features -> 4 layers -> guess in one kernel.  A warp owns
// 16 rows; the FP32 accumulator tiles of a layer (m16n8) are, two by two,
// exactly the A fragments (m16k16, BF16) of the next layer for the same
// lane, so activations never leave the registers.  Weights are read as B
// fragments pre-packed per (k-chunk, n-tile, lane) -- one coalesced 8-byte
// load per lane per mma -- from L1/L2, where all warps share them.  The
// products and their k order are those of gemm_bf16, so the guesses equal the
// layer-by-layer path's.
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// Packs W [K][Nn] (BF16) into B fragments: u32 index ((kc*NT + nt)*32 + lane)*2 + r.
__global__ void pack_b_fragments(const bf16 *W, int K, int Nn, uint32_t *out) {
  const int NT = Nn / 8, KC = K / 16;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)KC * NT * 64) return;
  const int r = (int)(i & 1), lane = (int)((i >> 1) & 31);
  const long long q = i >> 6;
  const int nt = (int)(q % NT), kc = (int)(q / NT);
  const int g = lane >> 2, t = lane & 3;
  const int k = kc * 16 + 2 * t + 8 * r, n = nt * 8 + g;
  const bf16 lo = W[(long long)k * Nn + n], hi = W[(long long)(k + 1) * Nn + n];
  out[i] = (uint32_t)(*reinterpret_cast<const uint16_t *>(&lo)) |
           ((uint32_t)(*reinterpret_cast<const uint16_t *>(&hi)) << 16);
}

struct FusedMLP {
  const uint2 *w1, *w2, *w3, *w4;  // packed B fragments per layer
  const float *b1, *b2, *b3, *b4;  // FP32 biases
  const float *fmu, *fisd, *tmu, *tsd;
};

// One hidden layer of 256 -> 256 for the warp's 16 rows: A fragments in ain
// (16 k-chunks x 4), GELU activations out as the next A fragments.
__device__ __forceinline__ void hidden_layer(const uint32_t (&ain)[16][4], uint32_t (&aout)[16][4],
                                             const uint2 *__restrict__ w, const float *__restrict__ b, int lane) {
  const int t = lane & 3;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int kc = 0; kc < 16; ++kc) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const uint2 bb = __ldg(&w[(kc * 32 + half * 16 + j) * 32 + lane]);
        const uint32_t bf[2] = {bb.x, bb.y};
        mma16816(acc[j], ain[kc], bf);
      }
    }
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      const int c0 = (half * 16 + j) * 8 + 2 * t, c1 = c0 + 8;
      const float b00 = __ldg(&b[c0]), b01 = __ldg(&b[c0 + 1]), b10 = __ldg(&b[c1]), b11 = __ldg(&b[c1 + 1]);
      uint32_t *o = aout[half * 8 + j / 2];
      o[0] = pack_bf16(gelu(acc[j][0] + b00), gelu(acc[j][1] + b01));
      o[1] = pack_bf16(gelu(acc[j][2] + b00), gelu(acc[j][3] + b01));
      o[2] = pack_bf16(gelu(acc[j + 1][0] + b10), gelu(acc[j + 1][1] + b11));
      o[3] = pack_bf16(gelu(acc[j + 1][2] + b10), gelu(acc[j + 1][3] + b11));
    }
  }
}

__global__ void __launch_bounds__(128) mlp_infer_fused(const CellArgs a, int N, int sorb, FusedMLP p, double *guess) {
  __shared__ float xs[4][16][kFeat + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const long long nc = a.ncells;
  const long long row0 = (blockIdx.x * 4LL + warp) * 16;
  if (row0 >= nc) return;
  // features of the warp's 16 rows, standardised as standardize() does
  if (lane < 16) {
    float x[kFeat];
    const long long cell = row0 + lane;
    if (cell < nc) {
      features_of(a, N, sorb, cell, x);
      for (int j = 0; j < kFeat; ++j) x[j] = (x[j] - p.fmu[j]) * p.fisd[j];
    } else {
      for (int j = 0; j < kFeat; ++j) x[j] = 0.f;
    }
    for (int j = 0; j < kFeat; ++j) xs[warp][lane][j] = x[j];
  }
  __syncwarp();
  uint32_t ax[4];
  ax[0] = pack_bf16(xs[warp][g][2 * t], xs[warp][g][2 * t + 1]);
  ax[1] = pack_bf16(xs[warp][g + 8][2 * t], xs[warp][g + 8][2 * t + 1]);
  ax[2] = pack_bf16(xs[warp][g][2 * t + 8], xs[warp][g][2 * t + 9]);
  ax[3] = pack_bf16(xs[warp][g + 8][2 * t + 8], xs[warp][g + 8][2 * t + 9]);
  // layer 1: 16 -> 256
  uint32_t h1[16][4], h2[16][4];
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
      const uint2 bb = __ldg(&p.w1[(half * 16 + j) * 32 + lane]);
      const uint32_t bf[2] = {bb.x, bb.y};
      mma16816(acc[j], ax, bf);
    }
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      const int c0 = (half * 16 + j) * 8 + 2 * t, c1 = c0 + 8;
      const float b00 = __ldg(&p.b1[c0]), b01 = __ldg(&p.b1[c0 + 1]), b10 = __ldg(&p.b1[c1]),
                  b11 = __ldg(&p.b1[c1 + 1]);
      uint32_t *o = h1[half * 8 + j / 2];
      o[0] = pack_bf16(gelu(acc[j][0] + b00), gelu(acc[j][1] + b01));
      o[1] = pack_bf16(gelu(acc[j][2] + b00), gelu(acc[j][3] + b01));
      o[2] = pack_bf16(gelu(acc[j + 1][0] + b10), gelu(acc[j + 1][1] + b11));
      o[3] = pack_bf16(gelu(acc[j + 1][2] + b10), gelu(acc[j + 1][3] + b11));
    }
  }
  hidden_layer(h1, h2, p.w2, p.b2, lane);  // layer 2
  hidden_layer(h2, h1, p.w3, p.b3, lane);  // layer 3
  // layer 4: 256 -> kOut (2 n-tiles), no activation
  float y[2][4];
#pragma unroll
  for (int j = 0; j < 2; ++j) y[j][0] = y[j][1] = y[j][2] = y[j][3] = 0.f;
#pragma unroll
  for (int kc = 0; kc < 16; ++kc)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const uint2 bb = __ldg(&p.w4[(kc * 2 + j) * 32 + lane]);
      const uint32_t bf[2] = {bb.x, bb.y};
      mma16816(y[j], h1[kc], bf);
    }
  // outputs -> alternative guess (as outputs_to_guess)
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = j * 8 + 2 * t + (q & 1);
      const long long cell = row0 + g + (q >= 2 ? 8 : 0);
      if (c < N && cell < nc) {
        const float z = y[j][q] + __ldg(&p.b4[c]);
        const double lm = (double)p.tmu[c] + (double)p.tsd[c] * (double)z;
        guess[c * nc + cell] = exp(fmin(fmax(lm, -700.0), 700.0));
      }
    }
}

__global__ void standardize(const float *X, const float *mu, const float *sd, bf16 *Xb, long long rows, int cols) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int c = (int)(i % cols);
  Xb[i] = __float2bfloat16((X[i] - mu[c]) * sd[c]);
}

// Predicted log-molalities of rows [r0, r0 + rows) -> alternative guess
// (SoA [N][ncells]), for the first N outputs.
__global__ void outputs_to_guess(const float *Y, int ldy, const float *mu, const float *sd, int N, long long rows,
                                 long long r0, long long ncells, double *guess) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  for (int j = 0; j < N; ++j) {
    const double lm = (double)mu[j] + (double)sd[j] * (double)Y[r * ldy + j];
    guess[j * ncells + r0 + r] = exp(fmin(fmax(lm, -700.0), 700.0));
  }
}

// Targets: converged molalities (SoA [N][M], double) -> standardised ln m ([M][N], float)
__global__ void targets_from_molal(const double *molal, long long M, int N, const float *mu, const float *sd,
                                   float *T) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= M) return;
  for (int j = 0; j < N; ++j) T[r * N + j] = (float)((log(molal[j * M + r]) - (double)mu[j]) / (double)sd[j]);
}

unsigned blocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <int EPI>
void gemm(cudaStream_t st, const bf16 *A, long long sam, long long sak, const bf16 *B, long long sbk, long long sbn,
          int M, int N, int K, const float *bias, float *Cf, bf16 *Cb, int ldc, int act) {
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  gemm_bf16<EPI><<<grid, 128, 0, st>>>(A, sam, sak, B, sbk, sbn, M, N, K, bias, Cf, Cb, ldc, act, K);
}

// C = A B over a long K (the weight gradients: K = the batch rows) split
// into `splits` slices of whole BK tiles, partials in `ws` (splits x M x N
// floats), summed in a fixed order into C (ldc = N).
void gemm_split_k(cudaStream_t st, const bf16 *A, long long sam, long long sak, const bf16 *B, long long sbk,
                  long long sbn, int M, int N, int K, float *C, float *ws, int splits) {
  int kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + BK - 1) / BK * BK;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);
  gemm_bf16<kEpiF32><<<grid, 128, 0, st>>>(A, sam, sak, B, sbk, sbn, M, N, K, nullptr, splits > 1 ? ws : C, nullptr,
                                           N, 0, kchunk);
  if (splits > 1) sum_splits<<<blocks((long long)M * N, 256), 256, 0, st>>>(ws, C, (long long)M * N, splits);
}

}  // namespace

// ---------------------------------------------------------------------------
struct Surrogate {
  int N = 0;           // outputs in use (network's primary species)
  int dims[kLayers + 1] = {kFeat, kHidden, kHidden, kHidden, kOut};
  // parameters (FP32 master, BF16 copy), gradients, Adam moments: one buffer each
  size_t woff[kLayers], boff[kLayers], nparam = 0;
  float *w = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
  bf16 *wb = nullptr;
  float *fmu = nullptr, *fsd = nullptr, *tmu = nullptr, *tsd = nullptr;  // device normalisation
  bool trained = false;
  // activations for a batch of `cap` rows (training) or one inference chunk
  long long cap = 0;
  bf16 *xb = nullptr, *hb[kLayers] = {}, *db[kLayers] = {};
  float *z[kLayers] = {}, *dz[kLayers] = {}, *y = nullptr, *dy = nullptr, *tgt = nullptr, *loss = nullptr;
  float *feat = nullptr;
  long long feat_cap = 0;
  double *guess = nullptr;
  long long guess_cap = 0;
  int steps = 0;
  uint32_t *wpk = nullptr;  // B-fragment packing of the BF16 weights (fused inference)
  float *ws = nullptr;      // split-K partials of the weight gradients (kSplits x 256 x 256)
  // tensor-core path of the dense layers: 0 = mma.sync (warp-level MMA, the
  // fused one-kernel inference), 1 = tcgen05.mma with tensor-memory accumulators
  int backend = 1;  // tcgen05 (PFCHEM_MLP_TCGEN05) unless the caller picks mma.sync
  int *uerr = nullptr;      // set by a tcgen05 kernel whose wait ran out
  bf16 *ubpk = nullptr;     // a layer's weights packed for the tcgen05 kernels (256 x 256)
  int sms = 0;
};
constexpr int kSplits = 16;  // weight-gradient GEMMs: K = batch rows split 16 ways

namespace {
void free_acts(Surrogate *s) {
  cudaFree(s->xb);
  for (int l = 0; l < kLayers; ++l) {
    cudaFree(s->hb[l]);
    cudaFree(s->db[l]);
    cudaFree(s->z[l]);
    cudaFree(s->dz[l]);
  }
  cudaFree(s->y);
  cudaFree(s->dy);
  cudaFree(s->tgt);
  s->xb = nullptr;
  for (int l = 0; l < kLayers; ++l) s->hb[l] = s->db[l] = nullptr, s->z[l] = s->dz[l] = nullptr;
  s->y = s->dy = s->tgt = nullptr;
  s->cap = 0;
}

cudaError_t ensure_acts(Surrogate *s, long long rows) {
  if (rows <= s->cap) return cudaSuccess;
  free_acts(s);
  cudaError_t e = cudaSuccess;
  e = cudaMalloc(&s->xb, rows * kFeat * sizeof(bf16));
  for (int l = 0; l < kLayers && e == cudaSuccess; ++l) {
    const int w = s->dims[l + 1];
    e = cudaMalloc(&s->hb[l], rows * w * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc(&s->db[l], rows * w * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc(&s->z[l], rows * w * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->dz[l], rows * w * sizeof(float));
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->y, rows * kOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->dy, rows * kOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->tgt, rows * kOut * sizeof(float));
  if (e == cudaSuccess) s->cap = rows;
  return e;
}

// forward over `rows` standardised inputs in s->xb; output FP32 in s->y
void forward(Surrogate *s, long long rows, cudaStream_t st, bool keep) {
  const bf16 *in = s->xb;
  for (int l = 0; l < kLayers; ++l) {
    const int K = s->dims[l], Nn = s->dims[l + 1];
    const bf16 *W = s->wb + s->woff[l];
    const float *b = s->w + s->boff[l];
    if (s->backend == 1 && umma_supports(Nn, K, true)) {
      if (l < kLayers - 1)
        umma_linear(st, in, rows, K, W, Nn, true, b, keep ? s->z[l] : nullptr, s->hb[l], kUmmaGeluE, s->uerr, s->sms,
                    s->ubpk);
      else
        umma_linear(st, in, rows, K, W, Nn, true, b, s->y, nullptr, kUmmaLinearE, s->uerr, s->sms, s->ubpk);
    } else if (l < kLayers - 1) {
      gemm<kEpiAct>(st, in, K, 1, W, Nn, 1, (int)rows, Nn, K, b, keep ? s->z[l] : nullptr, s->hb[l], Nn, 1);
    } else {
      gemm<kEpiF32>(st, in, K, 1, W, Nn, 1, (int)rows, Nn, K, b, s->y, nullptr, Nn, 0);
    }
    in = s->hb[l];
  }
}

// loss + gradients for `rows` rows (targets standardised in s->tgt, [rows][N])
void backward(Surrogate *s, long long rows, cudaStream_t st) {
  cudaMemsetAsync(s->grad, 0, s->nparam * sizeof(float), st);
  cudaMemsetAsync(s->loss, 0, sizeof(float), st);
  // output layer gradient: dY (FP32 in s->dy, BF16 in db[last])
  mse_loss<<<blocks(rows * kOut, 256), 256, 0, st>>>(s->y, s->tgt, s->dy, s->db[kLayers - 1], (int)rows, kOut,
                                                       s->N, s->loss);
  for (int l = kLayers - 1; l >= 0; --l) {
    const int K = s->dims[l], Nn = s->dims[l + 1];
    const bf16 *inp = (l == 0) ? s->xb : s->hb[l - 1];
    const bf16 *dZb = s->db[l];
    const float *dZf = (l == kLayers - 1) ? s->dy : s->dz[l];
    // dW[K x N] = inp^T [K x rows] . dZ [rows x N]
    gemm_split_k(st, inp, 1, K, dZb, Nn, 1, K, Nn, (int)rows, s->grad + s->woff[l], s->ws, kSplits);
    // db = column sums of dZ
    bias_grad<<<dim3(blocks(Nn, 128), 64), 128, 0, st>>>(dZf, s->grad + s->boff[l], (int)rows, Nn);
    if (l > 0) {
      // dH_{l-1} [rows x K] = dZ [rows x N] . W^T, W stored [K x N]
      const bf16 *W = s->wb + s->woff[l];
      if (s->backend == 1 && umma_supports(K, Nn, false))
        umma_linear(st, dZb, rows, Nn, W, K, false, nullptr, s->dz[l - 1], nullptr, kUmmaLinearE, s->uerr, s->sms,
                    s->ubpk);
      else
        gemm<kEpiF32>(st, dZb, Nn, 1, W, 1, Nn, (int)rows, K, Nn, nullptr, s->dz[l - 1], nullptr, K, 0);
      // through the GELU of layer l-1: dZ_{l-1} = dH * GELU'(Z_{l-1}) (in place in dz)
      gelu_backward<<<blocks(rows * K, 256), 256, 0, st>>>(s->dz[l - 1], s->z[l - 1], s->db[l - 1], s->dz[l - 1],
                                                           rows * K);
    }
  }
}
}  // namespace

Surrogate *surrogate_create(int N, uint64_t seed, std::string *err) {
  Surrogate *s = new Surrogate();
  s->N = N;
  size_t off = 0;
  for (int l = 0; l < kLayers; ++l) {
    s->woff[l] = off;
    off += (size_t)s->dims[l] * s->dims[l + 1];
    s->boff[l] = off;
    off += s->dims[l + 1];
  }
  s->nparam = off;
  // Kaiming-uniform weights (GELU ~ ReLU gain), zero biases, seeded
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kLayers; ++l) {
    const double bound = std::sqrt(6.0 / s->dims[l]) * (l == kLayers - 1 ? 0.5 : 1.0);
    std::uniform_real_distribution<double> U(-bound, bound);
    for (size_t i = 0; i < (size_t)s->dims[l] * s->dims[l + 1]; ++i) h[s->woff[l] + i] = (float)U(rng);
  }
  cudaError_t e = cudaMalloc(&s->w, off * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->grad, off * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->m1, off * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->m2, off * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->wb, off * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&s->wpk, off * sizeof(bf16));
  // split-K partials: the largest weight block is kHidden x kHidden
  if (e == cudaSuccess) e = cudaMalloc(&s->ws, (size_t)kSplits * kHidden * kHidden * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->fmu, 2 * kFeat * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->tmu, 2 * kOut * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->uerr, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s->ubpk, 256 * 256 * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMemset(s->uerr, 0, sizeof(int));
  if (e == cudaSuccess) e = umma_prepare();
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return nullptr;
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  s->fsd = s->fmu + kFeat;
  s->tsd = s->tmu + kOut;
  cudaMemcpy(s->w, h.data(), off * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(s->m1, 0, off * sizeof(float));
  cudaMemset(s->m2, 0, off * sizeof(float));
  to_bf16<<<blocks(off, 256), 256>>>(s->w, s->wb, off);
  std::vector<float> one(2 * kFeat, 0.f);
  for (int i = 0; i < kFeat; ++i) one[kFeat + i] = 1.f;
  cudaMemcpy(s->fmu, one.data(), 2 * kFeat * sizeof(float), cudaMemcpyHostToDevice);
  std::vector<float> onet(2 * kOut, 0.f);
  for (int i = 0; i < kOut; ++i) onet[kOut + i] = 1.f;
  cudaMemcpy(s->tmu, onet.data(), 2 * kOut * sizeof(float), cudaMemcpyHostToDevice);
  cudaDeviceSynchronize();
  return s;
}

void surrogate_destroy(Surrogate *s) {
  if (!s) return;
  free_acts(s);
  cudaFree(s->w);
  cudaFree(s->grad);
  cudaFree(s->m1);
  cudaFree(s->m2);
  cudaFree(s->wb);
  cudaFree(s->wpk);
  cudaFree(s->ws);
  cudaFree(s->uerr);
  cudaFree(s->ubpk);
  cudaFree(s->fmu);
  cudaFree(s->tmu);
  cudaFree(s->loss);
  cudaFree(s->feat);
  cudaFree(s->guess);
  delete s;
}

size_t surrogate_nparam(const Surrogate *s) { return s->nparam; }

cudaError_t surrogate_features(const DevNet &n, const CellArgs &a, float *X, cudaStream_t st) {
  cell_features<<<blocks(a.ncells, 128), 128, 0, st>>>(a, n.N, (n.Nix + n.Nsr) > 0, X);
  return cudaGetLastError();
}

// Sets the feature/target standardisation (host arrays: mean[kFeat], inv_std[kFeat], tmean[N], tstd[N]).
void surrogate_set_norm(Surrogate *s, const float *fmu, const float *fisd, const float *tmu, const float *tsd) {
  std::vector<float> f(2 * kFeat), t(2 * kOut, 0.f);
  for (int i = 0; i < kFeat; ++i) {
    f[i] = fmu[i];
    f[kFeat + i] = fisd[i];
  }
  for (int i = 0; i < kOut; ++i) t[kOut + i] = 1.f;
  for (int i = 0; i < s->N; ++i) {
    t[i] = tmu[i];
    t[kOut + i] = tsd[i];
  }
  cudaMemcpy(s->fmu, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(s->tmu, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice);
}

// One training step on `rows` raw feature rows X (device, [rows][kFeat]) and
// standardised targets T (device, [rows][N]).  Returns the mean loss (after
// the step's forward pass) when `sync`.
float surrogate_train_step(Surrogate *s, const float *X, const float *T, long long rows, float lr, float wd,
                           cudaStream_t st, bool sync, cudaError_t *err) {
  *err = ensure_acts(s, rows);
  if (*err != cudaSuccess) return NAN;
  standardize<<<blocks(rows * kFeat, 256), 256, 0, st>>>(X, s->fmu, s->fsd, s->xb, rows, kFeat);
  cudaMemcpyAsync(s->tgt, T, rows * s->N * sizeof(float), cudaMemcpyDeviceToDevice, st);
  forward(s, rows, st, true);
  backward(s, rows, st);
  s->steps += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - std::pow(b1, (float)s->steps), bc2 = 1.f - std::pow(b2, (float)s->steps);
  adamw<<<blocks(s->nparam, 256), 256, 0, st>>>(s->w, s->wb, s->grad, s->m1, s->m2, s->nparam, lr, b1, b2, 1e-8f, wd,
                                                 bc1, bc2);
  *err = cudaGetLastError();
  if (!sync) return 0.f;
  float l = 0.f;
  cudaMemcpyAsync(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return l;
}

// Loss and gradients (no update) for a batch: used to check the backward pass.
cudaError_t surrogate_gradients(Surrogate *s, const float *X, const float *T, long long rows, float *grad_host,
                                float *loss_host, cudaStream_t st) {
  cudaError_t e = ensure_acts(s, rows);
  if (e != cudaSuccess) return e;
  standardize<<<blocks(rows * kFeat, 256), 256, 0, st>>>(X, s->fmu, s->fsd, s->xb, rows, kFeat);
  cudaMemcpyAsync(s->tgt, T, rows * s->N * sizeof(float), cudaMemcpyDeviceToDevice, st);
  forward(s, rows, st, true);
  backward(s, rows, st);
  cudaMemcpyAsync(grad_host, s->grad, s->nparam * sizeof(float), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(loss_host, s->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
  return cudaStreamSynchronize(st);
}

cudaError_t surrogate_get_params(Surrogate *s, float *host) {
  return cudaMemcpy(host, s->w, s->nparam * sizeof(float), cudaMemcpyDeviceToHost);
}

cudaError_t surrogate_set_params(Surrogate *s, const float *host) {
  cudaError_t e = cudaMemcpy(s->w, host, s->nparam * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  to_bf16<<<blocks(s->nparam, 256), 256>>>(s->w, s->wb, s->nparam);
  return cudaDeviceSynchronize();
}

// Inference for a batch of cells: features -> MLP -> alternative guess
// (device SoA, [N][ncells]), processed in chunks of `chunk` rows.
constexpr long long kChunk = 1 << 18;  // inference rows per pass

// Allocates what surrogate_predict needs for `ncells` cells (call outside
// any stream capture).
cudaError_t surrogate_prepare(Surrogate *s, long long ncells) {
  cudaError_t e = ensure_acts(s, std::min(ncells, kChunk));
  if (e != cudaSuccess) return e;
  if (s->feat_cap < ncells) {
    cudaFree(s->feat);
    s->feat = nullptr;
    e = cudaMalloc(&s->feat, ncells * kFeat * sizeof(float));
    if (e != cudaSuccess) return e;
    s->feat_cap = ncells;
  }
  if (s->guess_cap < ncells) {
    cudaFree(s->guess);
    s->guess = nullptr;
    e = cudaMalloc(&s->guess, ncells * kOut * sizeof(double));
    if (e != cudaSuccess) return e;
    s->guess_cap = ncells;
  }
  return cudaSuccess;
}

double *surrogate_guess_buffer(Surrogate *s) { return s->guess; }

// Inference for a batch of cells: features -> MLP -> alternative guess into
// `guess` (device SoA, [N][ncells]; normally the surrogate's guess buffer).  Launch-only (no
// allocation, no synchronisation): capturable in a CUDA graph after
// surrogate_prepare.
// Refreshes the B-fragment packing of the current weights (140k values).
cudaError_t surrogate_pack(Surrogate *s, cudaStream_t st) {
  for (int l = 0; l < kLayers; ++l) {
    const int K = s->dims[l], Nn = s->dims[l + 1];
    pack_b_fragments<<<blocks((long long)(K / 16) * (Nn / 8) * 64, 256), 256, 0, st>>>(
        s->wb + s->woff[l], K, Nn, s->wpk + s->woff[l] / 2);  // woff is even: every K x N block is
  }
  return cudaGetLastError();
}

cudaError_t surrogate_predict_layers(Surrogate *s, const DevNet &n, const CellArgs &a, double *guess,
                                     cudaStream_t st);

cudaError_t surrogate_predict(Surrogate *s, const DevNet &n, const CellArgs &a, double *guess, cudaStream_t st,
                              bool pack) {
  const long long nc = a.ncells;
  // tcgen05 backend: layer by layer, each layer's weights resident in shared memory
  if (s->backend == 1) return surrogate_predict_layers(s, n, a, guess, st);
  if (pack) {
    cudaError_t e = surrogate_pack(s, st);
    if (e != cudaSuccess) return e;
  }
  uint32_t *pk[kLayers];
  for (int l = 0; l < kLayers; ++l) pk[l] = s->wpk + s->woff[l] / 2;
  FusedMLP p;
  p.w1 = reinterpret_cast<const uint2 *>(pk[0]);
  p.w2 = reinterpret_cast<const uint2 *>(pk[1]);
  p.w3 = reinterpret_cast<const uint2 *>(pk[2]);
  p.w4 = reinterpret_cast<const uint2 *>(pk[3]);
  p.b1 = s->w + s->boff[0];
  p.b2 = s->w + s->boff[1];
  p.b3 = s->w + s->boff[2];
  p.b4 = s->w + s->boff[3];
  p.fmu = s->fmu;
  p.fisd = s->fsd;
  p.tmu = s->tmu;
  p.tsd = s->tsd;
  mlp_infer_fused<<<blocks(nc, 64), 128, 0, st>>>(a, n.N, (n.Nix + n.Nsr) > 0, p, guess);
  return cudaGetLastError();
}

// The layer-by-layer inference path (GEMM kernels, HBM round trips between
// layers) into `guess`: kept to check the fused kernel against.
cudaError_t surrogate_predict_layers(Surrogate *s, const DevNet &n, const CellArgs &a, double *guess,
                                     cudaStream_t st) {
  const long long nc = a.ncells;
  cudaError_t e = surrogate_features(n, a, s->feat, st);
  if (e != cudaSuccess) return e;
  for (long long r0 = 0; r0 < nc; r0 += kChunk) {
    const long long rows = std::min(kChunk, nc - r0);
    standardize<<<blocks(rows * kFeat, 256), 256, 0, st>>>(s->feat + r0 * kFeat, s->fmu, s->fsd, s->xb, rows, kFeat);
    forward(s, rows, st, false);
    outputs_to_guess<<<blocks(rows, 128), 128, 0, st>>>(s->y, kOut, s->tmu, s->tsd, n.N, rows, r0, nc, guess);
  }
  return cudaGetLastError();
}

// Standardised targets from converged molalities (device SoA [N][M]) into T [M][N].
cudaError_t surrogate_targets(Surrogate *s, const double *molal, long long M, float *T, cudaStream_t st) {
  targets_from_molal<<<blocks(M, 128), 128, 0, st>>>(molal, M, s->N, s->tmu, s->tsd, T);
  return cudaGetLastError();
}

int surrogate_nfeat() { return kFeat; }
void surrogate_mark_trained(Surrogate *s, bool t) { s->trained = t; }
bool surrogate_trained(const Surrogate *s) { return s->trained; }
void surrogate_set_backend(Surrogate *s, int backend) { s->backend = backend; }
int surrogate_backend(const Surrogate *s) { return s->backend; }
// Reads and clears the tcgen05 kernels' timeout flag.
cudaError_t surrogate_check(Surrogate *s, bool *timed_out) {
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, s->uerr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h) e = cudaMemset(s->uerr, 0, sizeof(int));
  *timed_out = h != 0;
  return e;
}
// True when surrogate_predict can run on `ncells` cells without allocating.
bool surrogate_ready(const Surrogate *s, long long ncells) {
  return s->cap >= std::min(ncells, kChunk) && s->feat_cap >= ncells && s->guess_cap >= ncells;
}

}  // namespace pfchem
