// pfchem_umma.cu -- the warm-start MLP's dense layers on the 5th-generation
// tensor cores: tcgen05.mma (BF16 operands, FP32 accumulation in tensor
// memory), issued by one thread per CTA, completion signalled through an
// mbarrier, the accumulator read back with tcgen05.ld for a fused epilogue.
//
// C[rows x N] = X[rows x K] . B + bias, with B the layer's weights: stored
// K x N (n contiguous: the forward pass, X W) or N x K (k contiguous: the
// backward pass, dZ W^T).  A persistent grid of one CTA per SM keeps the
// whole B (up to 256 x 256 BF16, 128 KB) in shared memory and streams
// 128-row tiles of X through it: per tile the rows are staged into shared
// memory, K/16 MMAs of 128 x N x 16 accumulate into N tensor-memory columns,
// and the 128 threads read one row each (32x32b, 16 columns at a time) to
// add the bias, apply GELU and store BF16 and/or FP32.
//
// Operand layout: the canonical K-major layout without swizzle -- core
// matrices of 8 rows x 16 bytes stored contiguously, the next core matrix
// along K 128 bytes on, the next 8-row group (K/8)*128 bytes on; the shared
// memory descriptors carry those two strides.  Every wait is bounded: past
// its limit a CTA raises the error flag, skips its remaining tiles and still
// frees its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pfchem {

using bf16u = __nv_bfloat16;

enum { kUmmaGelu = 0, kUmmaLinear = 1 };

namespace {

__device__ __forceinline__ uint32_t u_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float u_gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

// shared-memory matrix descriptor, K-major, no swizzle (bits 46-48 = 0b001)
__device__ __forceinline__ uint64_t u_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t u_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool u_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

template <int N, int K, bool WKN>
__global__ void __launch_bounds__(128) umma_linear_kernel(const bf16u *__restrict__ X, long long rows,
                                                          const bf16u *__restrict__ W, const float *__restrict__ bias,
                                                          float *Cf, bf16u *Cb, int epi, int *err) {
  constexpr int TM = 128;
  constexpr int BBYTES = N * K * 2, ABYTES = TM * K * 2;
  constexpr int NCOL = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t *Bs = sm;
  uint8_t *As = sm + BBYTES;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + BBYTES + ABYTES);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + BBYTES + ABYTES + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(u_smem(tslot)), "n"(NCOL)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(u_smem(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // B (N rows, K contiguous) in core matrices: (n/8, k/8) at ((n/8)*(K/8) + k/8)*128, row n%8 at *16
  if (WKN) {  // stored K x N: 8 consecutive n per 16-byte load, scattered down a core-matrix column
    for (int e = tid; e < K * (N / 8); e += 128) {
      const int k = e / (N / 8), n0 = (e % (N / 8)) * 8;
      uint4 v = *reinterpret_cast<const uint4 *>(W + (size_t)k * N + n0);
      const bf16u *h = reinterpret_cast<const bf16u *>(&v);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int n = n0 + q;
        *reinterpret_cast<bf16u *>(Bs + ((n >> 3) * (K / 8) + (k >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2) = h[q];
      }
    }
  } else {  // stored N x K: one 16-byte load is one core-matrix row
    for (int e = tid; e < N * (K / 8); e += 128) {
      const int n = e / (K / 8), c = e % (K / 8);
      *reinterpret_cast<uint4 *>(Bs + ((n >> 3) * (K / 8) + c) * 128 + (n & 7) * 16) =
          *reinterpret_cast<const uint4 *>(W + (size_t)n * K + c * 8);
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  constexpr uint32_t idesc = u_idesc(TM, N);
  uint32_t phase = 0;
  bool ok = true;
  for (long long tile = blockIdx.x; tile * TM < rows; tile += gridDim.x) {
    const long long m0 = tile * TM;
    for (int e = tid; e < TM * (K / 8); e += 128) {
      const int m = e / (K / 8), c = e % (K / 8);
      uint4 v = make_uint4(0, 0, 0, 0);
      if (m0 + m < rows) v = *reinterpret_cast<const uint4 *>(X + (size_t)(m0 + m) * K + c * 8);
      *reinterpret_cast<uint4 *>(As + ((m >> 3) * (K / 8) + c) * 128 + (m & 7) * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
#pragma unroll 1
      for (int ks = 0; ks < K / 16; ++ks) {
        const uint64_t ad = u_desc(u_smem(As) + ks * 256, 128, (K / 8) * 128);
        const uint64_t bd = u_desc(u_smem(Bs) + ks * 256, 128, (K / 8) * 128);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(u_smem(mbar))
                   : "memory");
    }
    if (!u_wait(u_smem(mbar), phase)) {
      ok = false;
      if (tid == 0) atomicExch(err, 1);
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const long long row = m0 + tid;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < rows && ok) {
        float z[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) z[q] = __uint_as_float(r[q]) + (bias ? bias[c0 + q] : 0.f);
        if (Cf) {
          float4 *o = reinterpret_cast<float4 *>(Cf + (size_t)row * N + c0);
#pragma unroll
          for (int q = 0; q < 4; ++q) o[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        }
        if (Cb) {
          uint32_t p[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float a = epi == kUmmaGelu ? u_gelu(z[2 * q]) : z[2 * q];
            const float b = epi == kUmmaGelu ? u_gelu(z[2 * q + 1]) : z[2 * q + 1];
            const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
            p[q] = *reinterpret_cast<const uint32_t *>(&h);
          }
          uint4 *o = reinterpret_cast<uint4 *>(Cb + (size_t)row * N + c0);
          o[0] = make_uint4(p[0], p[1], p[2], p[3]);
          o[1] = make_uint4(p[4], p[5], p[6], p[7]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) break;
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(NCOL) : "memory");
}

template <int N, int K, bool WKN>
cudaError_t umma_launch_t(cudaStream_t st, const bf16u *X, long long rows, const bf16u *W, const float *bias,
                          float *Cf, bf16u *Cb, int epi, int *err, int grid) {
  // the shared-memory limit was raised by umma_prepare
  const size_t shm = (size_t)N * K * 2 + 128 * (size_t)K * 2 + 16;
  const long long tiles = (rows + 127) / 128;
  const int g = (int)(tiles < grid ? tiles : grid);
  umma_linear_kernel<N, K, WKN><<<g, 128, shm, st>>>(X, rows, W, bias, Cf, Cb, epi, err);
  return cudaGetLastError();
}

}  // namespace

// Raises the kernels' shared-memory limit (call outside any stream capture).
cudaError_t umma_prepare() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, size_t shm) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  };
  set((const void *)umma_linear_kernel<256, 16, true>, 256 * 16 * 2 + 128 * 16 * 2 + 16);
  set((const void *)umma_linear_kernel<256, 256, true>, 256 * 256 * 2 + 128 * 256 * 2 + 16);
  set((const void *)umma_linear_kernel<16, 256, true>, 16 * 256 * 2 + 128 * 256 * 2 + 16);
  set((const void *)umma_linear_kernel<256, 16, false>, 256 * 16 * 2 + 128 * 16 * 2 + 16);
  set((const void *)umma_linear_kernel<256, 256, false>, 256 * 256 * 2 + 128 * 256 * 2 + 16);
  return e;
}

// Whether umma_linear takes this (N, K, layout).
bool umma_supports(int N, int K, bool w_kn) {
  if (w_kn) return (N == 256 && (K == 16 || K == 256)) || (N == 16 && K == 256);
  return N == 256 && (K == 16 || K == 256);
}

// C = X[rows x K] . B + bias: B from W stored K x N (w_kn) or N x K; with
// Cb, epi kUmmaGelu stores BF16 GELU(C) and kUmmaLinear BF16 C; with Cf the
// FP32 C.  `err` (device int) is set if a CTA's wait ran out.  One CTA per SM.
cudaError_t umma_linear(cudaStream_t st, const bf16u *X, long long rows, int K, const bf16u *W, int N, bool w_kn,
                        const float *bias, float *Cf, bf16u *Cb, int epi, int *err, int sms) {
  if (rows <= 0) return cudaSuccess;
  if (w_kn) {
    if (N == 256 && K == 16) return umma_launch_t<256, 16, true>(st, X, rows, W, bias, Cf, Cb, epi, err, sms);
    if (N == 256 && K == 256) return umma_launch_t<256, 256, true>(st, X, rows, W, bias, Cf, Cb, epi, err, sms);
    if (N == 16 && K == 256) return umma_launch_t<16, 256, true>(st, X, rows, W, bias, Cf, Cb, epi, err, sms);
  } else {
    if (N == 256 && K == 16) return umma_launch_t<256, 16, false>(st, X, rows, W, bias, Cf, Cb, epi, err, sms);
    if (N == 256 && K == 256) return umma_launch_t<256, 256, false>(st, X, rows, W, bias, Cf, Cb, epi, err, sms);
  }
  return cudaErrorInvalidValue;
}

}  // namespace pfchem
