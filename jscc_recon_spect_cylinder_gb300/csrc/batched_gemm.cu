// Multi-instance (batched) SC OSEM on the 5th-generation tensor cores.
//
// N independent reconstructions that share one system matrix A (Poisson realisations or
// count levels of one geometry) turn the per-instance projector passes into two GEMMs per
// subset: F = A_s X (bins x instances) and W = A_s^T Q (voxels x instances). Both are
// computed by one kernel, C = P R^T with P [M x K] and R [Nr x K] both K-major BF16:
//   forward: P = A_s (subset rows of the bin-permuted matrix), R = images
//   back:    P = A^T restricted to the subset's bin columns (a stored transposed copy of the
//            permuted matrix, so both operands stay K-major), R = ratios
// The FP32 images and ratios enter as BF16 hi / lo pairs (v = hi + lo, ~16 significant
// bits), stacked as 2 Np rows of R, so the tensor-core product keeps FP32-level accuracy in
// the instance vectors while A is streamed from HBM once per pass for all instances.
//
// GEMM kernel (one 128-thread CTA per 128-row tile and K split):
//   * operands staged into shared memory by cp.async in the no-swizzle K-major core-matrix
//     layout (8 rows x 16 bytes per core matrix, core matrices K-fastest), zero-filled past
//     the matrix edges, 4-stage ring;
//   * one elected thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128,
//     N = Nr) into a TMEM accumulator of Nr columns and commits each stage to an mbarrier,
//     which releases the stage for the next cp.async round;
//   * epilogue: each warp reads its 32 TMEM lanes with tcgen05.ld and writes FP32 rows.
//   Every wait is bounded; a wait that gives up is counted (jscc_take_wait_timeout_count
//   does not see it: jscc_take_gemm_timeout_count does) and the CTA still frees its TMEM.
#include "jscc_common.cuh"

namespace jscc {

constexpr int kGM = 128;          // tile rows = MMA M
constexpr int kGK = 64;           // K per stage (128 bytes of BF16 per row)
constexpr int kGStages = 4;
constexpr int kGThreads = 128;
constexpr uint32_t kGemmPolls = 1u << 22;

__device__ unsigned int g_gemm_timeout_count = 0;

// Byte offset of element (r, k) of a [rows x 64] K-major tile: core matrix (r / 8, k / 8) of
// 8 rows x 16 bytes at ((r / 8) * 8 + k / 8) * 128, row r % 8 at 16-byte steps inside it.
// Adjacent core matrices along K are 128 bytes apart (leading byte offset), adjacent 8-row
// groups 1024 bytes (stride byte offset).
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)(((((r >> 3) << 3) + (k >> 3))) << 7) + (uint32_t)((r & 7) << 4) + (uint32_t)((k & 7) << 1);
}
constexpr uint32_t kLBO = 128;
constexpr uint32_t kSBO = 1024;

// tcgen05 shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading byte
// offset >> 4 (16-29), stride byte offset >> 4 (32-45), descriptor version 1 (46-47), base
// offset 0, no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor for kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int NR>
struct GemmCfg {
  static_assert(NR % 16 == 0 && NR >= 16 && NR <= 256, "MMA N for M = 128");
  static constexpr uint32_t kA = kGM * kGK * 2;
  static constexpr uint32_t kB = NR * kGK * 2;
  static constexpr uint32_t kStage = kA + kB;
  static constexpr uint32_t kTmemCols = NR <= 32 ? 32 : NR <= 64 ? 64 : NR <= 128 ? 128 : 256;
  static constexpr size_t kSmem = (size_t)kGStages * kStage + 64 + 1024;  // + barriers, TMEM slot, alignment
};

// out[split][m][n] = sum_{k in split} P[m, k] R[n, k]   (rows m < M, n < nr; FP32)
template <int NR>
__global__ void __launch_bounds__(kGThreads, 1)
bf16_gemm_nt_kernel(const __nv_bfloat16* __restrict__ P, int64_t ldp, const __nv_bfloat16* __restrict__ R,
                    int64_t ldr, int64_t M, int nr, int64_t K, int64_t k_per_split, float* __restrict__ out,
                    int64_t ldo, int64_t split_stride) {
  using C = GemmCfg<NR>;
  extern __shared__ uint8_t gsm_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(gsm_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kGStages * C::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kGStages);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kGM;
  const int64_t kb = (int64_t)blockIdx.y * k_per_split;
  const int64_t ke = (kb + k_per_split) < K ? (kb + k_per_split) : K;
  const int nk = ke > kb ? (int)((ke - kb + kGK - 1) / kGK) : 0;

  if (tid == 0) {
    for (int s = 0; s < kGStages; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sbase = smem_u32(smem);

  auto load_tile = [&](int t) {
    const int s = t % kGStages;
    const uint32_t a_base = sbase + s * C::kStage, b_base = a_base + C::kA;
    const int64_t k0 = kb + (int64_t)t * kGK;
    for (int c = tid; c < kGM * 8; c += kGThreads) {
      const int r = c >> 3, kc = (c & 7) << 3;
      const int64_t gr = m0 + r, gk = k0 + kc;
      const bool ok = gr < M && gk < ke;  // K and the split boundaries are multiples of 8
      cp_async16(a_base + tile_off(r, kc), ok ? (const void*)(P + gr * ldp + gk) : (const void*)P, ok ? 16u : 0u);
    }
    for (int c = tid; c < NR * 8; c += kGThreads) {
      const int r = c >> 3, kc = (c & 7) << 3;
      const int64_t gk = k0 + kc;
      const bool ok = r < nr && gk < ke;
      cp_async16(b_base + tile_off(r, kc), ok ? (const void*)(R + (int64_t)r * ldr + gk) : (const void*)R,
                 ok ? 16u : 0u);
    }
  };

  constexpr uint32_t idesc = umma_idesc(kGM, NR);
  bool failed = false;
#pragma unroll 1
  for (int t = 0; t < kGStages - 1; ++t) {
    if (t < nk) load_tile(t);
    cp_async_commit();
  }
#pragma unroll 1
  for (int t = 0; t < nk; ++t) {
    const int tn = t + kGStages - 1;
    bool bad = false;
    if (tn < nk) {
      if (t >= 1) {
        // stage (t - 1) % S is refilled: the MMAs of tile t - 1 must have read it
        const int sp = (t - 1) % kGStages;
        bad = !mbar_wait_bounded(&bars[sp], (uint32_t)(((t - 1) / kGStages) & 1), kGemmPolls);
      }
      if (!bad) load_tile(tn);
    }
    cp_async_commit();
    cp_async_wait<kGStages - 1>();
    fence_proxy_async_smem();
    if (__syncthreads_or(bad)) {
      failed = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a_base = sbase + (t % kGStages) * C::kStage, b_base = a_base + C::kA;
#pragma unroll
      for (int kk = 0; kk < kGK / 16; ++kk)  // K = 16 per MMA: two core matrices = 256 bytes
        tc_mma(tmem, umma_desc(a_base + kk * 256), umma_desc(b_base + kk * 256), idesc, (t > 0 || kk > 0) ? 1u : 0u);
      tc_commit(&bars[t % kGStages]);
    }
  }
  cp_async_wait<0>();
  // the last commit covers every MMA issued before it
  bool done = true;
  if (nk > 0 && !failed) done = mbar_wait_bounded(&bars[(nk - 1) % kGStages], (uint32_t)(((nk - 1) / kGStages) & 1),
                                                  kGemmPolls);
  const bool ok = __syncthreads_and(done && !failed);
  tc_fence_after();
  const int64_t row = m0 + warp * 32 + lane;
  float* orow = out + (int64_t)blockIdx.y * split_stride + row * ldo;
  if (ok) {
#pragma unroll 1
    for (int c0 = 0; c0 < NR; c0 += 32) {
      float v[32];
      if (nk > 0) {
        tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = 0.f;
      }
      if (row < M) {
#pragma unroll
        for (int i = 0; i < 32; ++i)
          if (c0 + i < nr) orow[c0 + i] = v[i];
      }
    }
  } else if (tid == 0) {
    atomicAdd(&g_gemm_timeout_count, 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::kTmemCols) : "memory");
  }
}

// out[m][n] = sum_s part[s][m][n] (fixed split order)
__global__ void gemm_split_reduce_kernel(const float* __restrict__ part, int splits, int64_t split_stride, int64_t M,
                                         int nr, float* __restrict__ out, int64_t ldo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < M * nr; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = t / nr;
    const int n = (int)(t % nr);
    float acc = 0.f;
    for (int s = 0; s < splits; ++s) acc += part[(int64_t)s * split_stride + m * nr + n];
    out[m * ldo + n] = acc;
  }
}

// ------------------------------------------------------------------ batch helpers
__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// xs[n][v] = hi(x[n][v]), xs[np + n][v] = lo(x[n][v]); rows n >= n_inst are zero.
__global__ void batch_split_kernel(const float* __restrict__ x, int64_t ldx, int n_inst, int np, int64_t V,
                                   __nv_bfloat16* __restrict__ xs, int64_t ldxs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)np * V;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / V);
    const int64_t v = t % V;
    __nv_bfloat16 hi = __float2bfloat16_rn(0.f), lo = hi;
    if (n < n_inst) split_bf16(x[n * ldx + v], hi, lo);
    xs[(int64_t)n * ldxs + v] = hi;
    xs[(int64_t)(np + n) * ldxs + v] = lo;
  }
}

// f[b][n] = F[b][n] + F[b][np + n] (forward GEMM columns: hi and lo image halves);
// q = y[n][b0 + b] / f; qs[n][b] = hi(q), qs[np + n][b] = lo(q). Optionally f_out[n][b] = f.
__global__ void batch_ratio_kernel(const float* __restrict__ F, int64_t ldf, const float* __restrict__ y, int64_t ldy,
                                   int64_t b0, int64_t nb, int n_inst, int np, __nv_bfloat16* __restrict__ qs,
                                   int64_t ldqs, float* __restrict__ f_out, int64_t ldfo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)np * nb;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / nb);
    const int64_t b = t % nb;
    __nv_bfloat16 hi = __float2bfloat16_rn(0.f), lo = hi;
    if (n < n_inst) {
      const float f = F[b * ldf + n] + F[b * ldf + np + n];
      if (f_out) f_out[(int64_t)n * ldfo + b] = f;
      split_bf16(__fdiv_rn(y[(int64_t)n * ldy + b0 + b], f), hi, lo);
    }
    qs[(int64_t)n * ldqs + b] = hi;
    qs[(int64_t)(np + n) * ldqs + b] = lo;
  }
}

// w[n][v] = scale * (W[v][n] + W[v][np + n]) (+= into w_out when accumulate).
__global__ void batch_weight_kernel(const float* __restrict__ W, int64_t ldw, int64_t V, int n_inst, int np,
                                    float scale, float* __restrict__ w_out, int64_t ldwo, int accumulate) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n_inst * V;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / V);
    const int64_t v = t % V;
    const float w = __fmul_rn(scale, __fadd_rn(W[v * ldw + n], W[v * ldw + np + n]));
    float* dst = w_out + (int64_t)n * ldwo + v;
    *dst = accumulate ? __fadd_rn(*dst, w) : w;
  }
}

// x[n][v] = x[n][v] * (W[v][n] + W[v][np + n]) / s[v] (the plain EM update of
// recon_osem_plane.py:54 per instance), and the updated image's hi / lo BF16 pair into xs
// (the next subset's forward operand) when xs is non-NULL.
__global__ void batch_em_kernel(const float* __restrict__ W, int64_t ldw, int64_t V, int n_inst, int np,
                                float* __restrict__ x, int64_t ldx, const float* __restrict__ s,
                                __nv_bfloat16* __restrict__ xs, int64_t ldxs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n_inst * V;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / V);
    const int64_t v = t % V;
    const float w = __fadd_rn(W[v * ldw + n], W[v * ldw + np + n]);
    float* px = x + (int64_t)n * ldx + v;
    const float xn = __fdiv_rn(__fmul_rn(*px, w), s[v]);
    *px = xn;
    if (xs) {
      __nv_bfloat16 hi, lo;
      split_bf16(xn, hi, lo);
      xs[(int64_t)n * ldxs + v] = hi;
      xs[(int64_t)(np + n) * ldxs + v] = lo;
    }
  }
}

}  // namespace jscc

using namespace jscc;

namespace {

template <int NR>
int launch_gemm(const __nv_bfloat16* P, int64_t ldp, const __nv_bfloat16* R, int64_t ldr, int64_t M, int nr, int64_t K,
                int splits, float* out, int64_t ldo, float* part, cudaStream_t st) {
  using C = GemmCfg<NR>;
  static bool attr_set = false;  // per process; the attribute is a property of the function
  if (!attr_set) {
    JSCC_CUDA_CHECK(cudaFuncSetAttribute(bf16_gemm_nt_kernel<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)C::kSmem));
    attr_set = true;
  }
  int64_t kps = (K + splits - 1) / splits;
  kps = (kps + kGK - 1) / kGK * kGK;
  if (kps < kGK) kps = kGK;  // K = 0: one split whose tiles write zeros
  int64_t used = (K + kps - 1) / kps;
  if (used < 1) used = 1;
  dim3 grid((unsigned)((M + kGM - 1) / kGM), (unsigned)used);
  float* dst = used > 1 ? part : out;
  const int64_t ldd = used > 1 ? nr : ldo;
  const int64_t sstride = used > 1 ? M * nr : 0;
  JSCC_TIMED("bf16_gemm_nt", st,
             (bf16_gemm_nt_kernel<NR><<<grid, kGThreads, C::kSmem, st>>>(P, ldp, R, ldr, M, nr, K, kps, dst, ldd,
                                                                        sstride)));
  JSCC_LAUNCH_CHECK();
  if (used > 1) {
    int64_t blocks = (M * nr + 255) / 256;
    if (blocks > (int64_t)num_sms() * 8) blocks = (int64_t)num_sms() * 8;
    JSCC_TIMED("gemm_split_reduce", st,
               (gemm_split_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part, (int)used, sstride, M, nr, out, ldo)));
    JSCC_LAUNCH_CHECK();
  }
  return JSCC_OK;
}

int64_t grid_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (b > cap) b = cap;
  return b < 1 ? 1 : b;
}

}  // namespace

extern "C" {

size_t jscc_bf16_gemm_workspace_bytes(int64_t M, int32_t nr, int64_t K, int32_t k_splits) {
  if (k_splits <= 1) return 256;
  return align_up((size_t)k_splits * (size_t)(M > 0 ? M : 1) * (size_t)(nr > 0 ? nr : 1) * sizeof(float), 256) + 256;
}

int jscc_bf16_gemm_nt(const void* P, int64_t ldp, const void* R, int64_t ldr, int64_t M, int32_t nr, int64_t K,
                      int32_t k_splits, float* out, int64_t ldo, void* workspace, size_t workspace_bytes,
                      void* stream) {
  JSCC_REQUIRE(M >= 0 && K >= 0, "jscc_bf16_gemm_nt: negative size");
  JSCC_REQUIRE(nr >= 1 && nr <= 256, "jscc_bf16_gemm_nt: nr = %d outside [1, 256]", nr);
  JSCC_REQUIRE(k_splits >= 1 && k_splits <= 64, "jscc_bf16_gemm_nt: k_splits = %d outside [1, 64]", k_splits);
  if (M == 0) return JSCC_OK;
  JSCC_REQUIRE(out && ((P && R) || K == 0), "jscc_bf16_gemm_nt: null pointer argument");
  JSCC_REQUIRE(K % 8 == 0 && (K == 0 || (ldp % 8 == 0 && ldr % 8 == 0)),
               "jscc_bf16_gemm_nt: K, ldp and ldr must be multiples of 8");
  JSCC_REQUIRE(ldp >= K && ldr >= K && ldo >= nr, "jscc_bf16_gemm_nt: leading dimension too small");
  JSCC_REQUIRE(reinterpret_cast<uintptr_t>(P) % 16 == 0 && reinterpret_cast<uintptr_t>(R) % 16 == 0,
               "jscc_bf16_gemm_nt: P and R must be 16-byte aligned");
  JSCC_REQUIRE(k_splits == 1 || (workspace != nullptr &&
                                 workspace_bytes >= jscc_bf16_gemm_workspace_bytes(M, nr, K, k_splits)),
               "jscc_bf16_gemm_nt: workspace too small");
  const auto* p = static_cast<const __nv_bfloat16*>(P);
  const auto* r = static_cast<const __nv_bfloat16*>(R);
  float* part = static_cast<float*>(workspace);
  cudaStream_t st = as_stream(stream);
  if (nr <= 32) return launch_gemm<32>(p, ldp, r, ldr, M, nr, K, k_splits, out, ldo, part, st);
  if (nr <= 64) return launch_gemm<64>(p, ldp, r, ldr, M, nr, K, k_splits, out, ldo, part, st);
  if (nr <= 128) return launch_gemm<128>(p, ldp, r, ldr, M, nr, K, k_splits, out, ldo, part, st);
  return launch_gemm<256>(p, ldp, r, ldr, M, nr, K, k_splits, out, ldo, part, st);
}

int jscc_batch_split(const float* x, int64_t ldx, int32_t n_inst, int32_t np, int64_t V, void* xs, int64_t ldxs,
                     void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && V >= 0, "jscc_batch_split: bad sizes");
  if (np == 0 || V == 0) return JSCC_OK;
  JSCC_REQUIRE(xs && (x || n_inst == 0), "jscc_batch_split: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_split", st,
             (batch_split_kernel<<<(unsigned)grid_blocks((int64_t)np * V), 256, 0, st>>>(
                 x, ldx, n_inst, np, V, static_cast<__nv_bfloat16*>(xs), ldxs)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_batch_ratio(const float* F, int64_t ldf, const float* y, int64_t ldy, int64_t b0, int64_t nb, int32_t n_inst,
                     int32_t np, void* qs, int64_t ldqs, float* f_out, int64_t ldfo, void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && nb >= 0 && b0 >= 0, "jscc_batch_ratio: bad sizes");
  if (np == 0 || nb == 0) return JSCC_OK;
  JSCC_REQUIRE(F && y && qs, "jscc_batch_ratio: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_ratio", st,
             (batch_ratio_kernel<<<(unsigned)grid_blocks((int64_t)np * nb), 256, 0, st>>>(
                 F, ldf, y, ldy, b0, nb, n_inst, np, static_cast<__nv_bfloat16*>(qs), ldqs, f_out, ldfo)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_batch_weight(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np, float scale, float* w_out,
                      int64_t ldwo, int32_t accumulate, void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && V >= 0, "jscc_batch_weight: bad sizes");
  if (n_inst == 0 || V == 0) return JSCC_OK;
  JSCC_REQUIRE(W && w_out, "jscc_batch_weight: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_weight", st,
             (batch_weight_kernel<<<(unsigned)grid_blocks((int64_t)n_inst * V), 256, 0, st>>>(
                 W, ldw, V, n_inst, np, scale, w_out, ldwo, accumulate)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_batch_em(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np, float* x, int64_t ldx,
                  const float* s_map, void* xs, int64_t ldxs, void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && V >= 0, "jscc_batch_em: bad sizes");
  if (n_inst == 0 || V == 0) return JSCC_OK;
  JSCC_REQUIRE(W && x && s_map, "jscc_batch_em: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_em", st,
             (batch_em_kernel<<<(unsigned)grid_blocks((int64_t)n_inst * V), 256, 0, st>>>(
                 W, ldw, V, n_inst, np, x, ldx, s_map, static_cast<__nv_bfloat16*>(xs), ldxs)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_take_gemm_timeout_count(unsigned int* out) {
  JSCC_REQUIRE(out, "jscc_take_gemm_timeout_count: null pointer argument");
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_gemm_timeout_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_gemm_timeout_count, &zero, sizeof(zero)));
  *out = h;
  return JSCC_OK;
}

}  // extern "C"
