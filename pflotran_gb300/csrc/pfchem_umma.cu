// pfchem_umma.cu -- the warm-start MLP's dense layers on the 5th-generation
// tensor cores: tcgen05.mma (BF16 operands, FP32 accumulation in tensor
// memory), issued by one thread per CTA, completion signalled through an
// mbarrier, the accumulator read back with tcgen05.ld for a fused epilogue.
//
// C[rows x N] = X[rows x K] . B + bias, with B the layer's weights: stored
// K x N (n contiguous: the forward pass, X W) or N x K (k contiguous: the
// backward pass, dZ W^T), packed by a small kernel into the operand layout
// first.  A persistent grid of one CTA (16 warps) per SM keeps the whole B (up
// to 256 x 256 BF16, 128 KB) in shared memory and streams 128-row tiles of X
// through it: cp.async stages a tile into shared memory, K/16 MMAs of
// 128 x N x 16 accumulate into N tensor-memory columns, and while the next
// tile's copies are in flight the 16 warps read the accumulator (warp w: rows
// 32*(w%4).., a quarter w/4 of the columns, 16 columns at a time) to add the
// bias (held in shared memory), apply GELU and store BF16 and/or FP32.
//
// Operand layout: the canonical K-major layout without swizzle -- core
// matrices of 8 rows x 16 bytes stored contiguously, the next core matrix
// along K 128 bytes on, the next 8-row group (K/8)*128 bytes on; the shared
// memory descriptors carry those two strides.  Every wait is bounded: past
// its limit a CTA raises the error flag, skips its remaining tiles, waits for
// its copies and still frees its tensor memory.
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

// B packed once per call into the operand layout below, so that every CTA
// copies it as one contiguous block: chunk (n, k/8) -- 8 consecutive k of
// row n of B -- at ((n/8)*(K/8) + k/8)*128 + (n%8)*16 bytes.  W is R x C
// row-major; the forward pass (B[n][k] = W[k][n], W stored K x N) transposes,
// the backward pass (B = W, stored N x K) does not.
__global__ void umma_pack_kernel(const bf16u *__restrict__ W, int R, int C, int transpose, bf16u *__restrict__ out) {
  const int Nn = transpose ? C : R, K = transpose ? R : C, CPR = K / 8;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= Nn * CPR) return;
  const int r = e & 7, j = e >> 3, kc = j % CPR, n = (j / CPR) * 8 + r, k0 = kc * 8;
  __align__(16) bf16u v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = transpose ? W[(size_t)(k0 + q) * C + n] : W[(size_t)n * C + k0 + q];
  *reinterpret_cast<uint4 *>(out + (size_t)e * 8) = *reinterpret_cast<const uint4 *>(v);
}

__device__ __forceinline__ void u_cp16(uint32_t dst, const void *src, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

constexpr int kUThreads = 512;  // 16 warps: loads and epilogue; thread 0 issues the MMAs

// The A tile of rows [m0, m0 + 128) into shared memory with cp.async, zero
// rows past `rows`.  One warp instruction moves 8 rows x 4 chunks (K >= 32)
// or 16 rows x 2 chunks (K = 16): 512 contiguous bytes of shared memory (four
// core matrices, no bank conflicts) from whole 32-byte sectors of X.
template <int K>
__device__ __forceinline__ void u_load_a(uint8_t *As, const bf16u *__restrict__ X, long long m0, long long rows,
                                         int warp, int lane) {
  constexpr int CPR = K / 8, CW = CPR < 4 ? CPR : 4, RPW = 8 * (4 / CW), NCB = CPR / CW;
  constexpr int UNITS = (128 / RPW) * NCB;
  const int r = lane & 7, g = lane >> 3, coff = g % CW, rb = g / CW;
  const uint32_t base = u_smem(As);
#pragma unroll 4
  for (int u = warp; u < UNITS; u += kUThreads / 32) {
    const int m = (u / NCB) * RPW + rb * 8 + r, c = (u % NCB) * CW + coff;
    const bool in = m0 + m < rows;
    const bf16u *src = in ? X + (size_t)(m0 + m) * K + c * 8 : X;
    u_cp16(base + ((m >> 3) * CPR + c) * 128 + (m & 7) * 16, src, in ? 16u : 0u);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N, int K>
__global__ void __launch_bounds__(kUThreads, 1) umma_linear_kernel(const bf16u *__restrict__ X, long long rows,
                                                                   const bf16u *__restrict__ Bpk,
                                                                   const float *__restrict__ bias, float *Cf, bf16u *Cb,
                                                                   int epi, int *err) {
  constexpr int TM = 128;
  constexpr int BBYTES = N * K * 2, ABYTES = TM * K * 2;
  constexpr int NCOL = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t *Bs = sm;
  uint8_t *As = sm + BBYTES;
  float *bias_s = reinterpret_cast<float *>(sm + BBYTES + ABYTES);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + BBYTES + ABYTES + N * 4);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + BBYTES + ABYTES + N * 4 + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int c = tid; c < N; c += kUThreads) bias_s[c] = bias ? bias[c] : 0.f;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(u_smem(tslot)), "n"(NCOL)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(u_smem(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the packed B: one contiguous copy; then the first A tile
  for (int e = tid; e < BBYTES / 16; e += kUThreads) u_cp16(u_smem(Bs) + e * 16, Bpk + (size_t)e * 8, 16u);
  long long tile = blockIdx.x;
  if (tile * TM < rows) u_load_a<K>(As, X, tile * TM, rows, warp, lane);
  else asm volatile("cp.async.commit_group;" ::: "memory");
  constexpr uint32_t idesc = u_idesc(TM, N);
  uint32_t phase = 0;
  bool ok = true;
  // epilogue split: warp w reads TMEM lanes 32*(w%4).. (rows) and part w/4 of the columns
  // (a quarter of them; with N = 16 the first four warps take all 16)
  const int quarter = warp & 3, part = warp >> 2;
  constexpr int CW_EPI = N >= 64 ? N / 4 : N;
  const int c_begin = part * CW_EPI, c_end = (N >= 64 || part == 0) ? c_begin + CW_EPI : c_begin;
  for (; tile * TM < rows; tile += gridDim.x) {
    const long long m0 = tile * TM;
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tslot);
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
    // the MMAs have read the A tile: fetch the next one during the epilogue
    const long long next = tile + gridDim.x;
    if (ok && next * TM < rows) u_load_a<K>(As, X, next * TM, rows, warp, lane);
    const long long row = m0 + quarter * 32 + lane;
#pragma unroll 1
    for (int c0 = c_begin; c0 < c_end; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
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
        for (int q = 0; q < 16; ++q) z[q] = __uint_as_float(r[q]) + bias_s[c0 + q];
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
    // every TMEM read is done before the next tile's MMAs overwrite the accumulator
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) break;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tslot);
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(NCOL) : "memory");
  }
}

template <int N, int K>
constexpr size_t u_shm() {
  return (size_t)N * K * 2 + 128 * (size_t)K * 2 + (size_t)N * 4 + 16;
}

template <int N, int K>
cudaError_t umma_launch_t(cudaStream_t st, const bf16u *X, long long rows, const bf16u *Bpk, const float *bias,
                          float *Cf, bf16u *Cb, int epi, int *err, int grid) {
  // the shared-memory limit was raised by umma_prepare
  const long long tiles = (rows + 127) / 128;
  const int g = (int)(tiles < grid ? tiles : grid);
  umma_linear_kernel<N, K><<<g, kUThreads, u_shm<N, K>(), st>>>(X, rows, Bpk, bias, Cf, Cb, epi, err);
  return cudaGetLastError();
}

}  // namespace

// Raises the kernels' shared-memory limit (call outside any stream capture).
cudaError_t umma_prepare() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, size_t shm) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  };
  set((const void *)umma_linear_kernel<256, 16>, u_shm<256, 16>());
  set((const void *)umma_linear_kernel<256, 256>, u_shm<256, 256>());
  set((const void *)umma_linear_kernel<16, 256>, u_shm<16, 256>());
  return e;
}

// Whether umma_linear takes this (N, K, layout).
bool umma_supports(int N, int K, bool w_kn) {
  if (w_kn) return (N == 256 && (K == 16 || K == 256)) || (N == 16 && K == 256);
  return N == 256 && (K == 16 || K == 256);
}

// C = X[rows x K] . B + bias: B from W stored K x N (w_kn) or N x K, packed
// into `bpk` (N*K BF16 of device scratch) first; with Cb, epi kUmmaGelu stores
// BF16 GELU(C) and kUmmaLinear BF16 C; with Cf the FP32 C.  `err` (device int)
// is set if a CTA's wait ran out.  One CTA per SM.
cudaError_t umma_linear(cudaStream_t st, const bf16u *X, long long rows, int K, const bf16u *W, int N, bool w_kn,
                        const float *bias, float *Cf, bf16u *Cb, int epi, int *err, int sms, bf16u *bpk) {
  if (rows <= 0) return cudaSuccess;
  if (!umma_supports(N, K, w_kn) || !bpk) return cudaErrorInvalidValue;
  const int chunks = N * K / 8;
  umma_pack_kernel<<<(chunks + 255) / 256, 256, 0, st>>>(W, w_kn ? K : N, w_kn ? N : K, w_kn ? 1 : 0, bpk);
  if (N == 256 && K == 16) return umma_launch_t<256, 16>(st, X, rows, bpk, bias, Cf, Cb, epi, err, sms);
  if (N == 256 && K == 256) return umma_launch_t<256, 256>(st, X, rows, bpk, bias, Cf, Cb, epi, err, sms);
  return umma_launch_t<16, 256>(st, X, rows, bpk, bias, Cf, Cb, epi, err, sms);
}

}  // namespace pfchem
