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
// GEMM kernel (one 128-thread CTA per 128-row tile and K split, two CTAs per SM,
// warp-specialised):
//   * producer (warp 0, one thread): TMA tiled loads (cp.async.bulk.tensor, 128-byte swizzle)
//     of the P and R tiles of each 64-wide K step into a ring of shared-memory stages, each
//     completing on the stage's "full" mbarrier (expect-tx bytes);
//   * MMA issuer (warp 1, one thread): waits "full", issues tcgen05.mma (kind::f16, BF16 x
//     BF16 -> FP32, M = 128, N = Nr, K = 16 per instruction) into a TMEM accumulator of Nr
//     columns, and commits to the stage's "empty" mbarrier, which the producer waits for
//     before refilling it; a last commit signals the epilogue;
//   * epilogue (all four warps): each warp reads its 32 TMEM lanes with tcgen05.ld and writes
//     FP32 rows.
//   Every wait is bounded (jscc_set_wait_limit) and polls a CTA abort flag. A CTA that gives
//   up first waits, with a fixed bound of its own, for the work it already issued: the TMA
//   loads that the MMA issuer did not consume (they still write shared memory) and the MMAs
//   it committed (they still write TMEM and read shared memory). Only then is it counted
//   (jscc_take_gemm_timeout_count), skips the epilogue and frees its TMEM.
#include "jscc_common.cuh"

#include <cuda.h>

#include <atomic>
#include <cstring>

namespace jscc {

constexpr int kGM = 128;          // tile rows = MMA M
constexpr int kGK = 64;           // K per stage (128 bytes of BF16 per row)
constexpr int kGThreads = 128;
constexpr uint32_t kGemmPolls = 1u << 22;       // default bound of a role's wait
constexpr uint32_t kGemmDrainPolls = 1u << 24;  // bound of the drain after a give-up

__device__ unsigned int g_gemm_timeout_count = 0;
// Poll bound of the role waits, settable from the host (jscc_set_wait_limit): 0 makes every
// role wait give up at once, which exercises the give-up path with all copies completing.
__device__ uint32_t g_gemm_poll_limit = kGemmPolls;

// tcgen05 shared-memory matrix descriptor for a K-major tile written by TMA with 128-byte
// swizzle (rows of 64 BF16 = 128 bytes, 8-row atoms of 1024 bytes): start address >> 4
// (bits 0-13), leading byte offset 16 >> 4 (unused inside one swizzle row), stride byte
// offset 1024 >> 4 (32-45), descriptor version 1 (46-47), layout SWIZZLE_128B = 2 (61-63).
// A K = 16 slice starts 32 bytes further along the row.
__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// Instruction descriptor for kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
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

// Bounded wait that also gives up when another role of the CTA raised the abort flag.
__device__ __forceinline__ bool role_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          uint32_t polls) {
  for (uint32_t i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255) == 255 && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

template <int NR>
struct GemmCfg {
  static_assert(NR % 16 == 0 && NR >= 16 && NR <= 256, "MMA N for M = 128");
  static constexpr uint32_t kA = kGM * kGK * 2;  // 16 KB
  static constexpr uint32_t kB = NR * kGK * 2;
  static constexpr uint32_t kStage = kA + kB;
  // ~100 KB of stages: two CTAs per SM (their TMA rings interleave, so both grids of a
  // config-4 subset fit one wave of 2 x 152 CTAs)
  static constexpr int kStages = (100u * 1024u / kStage) < 8u ? (int)(100u * 1024u / kStage) : 8;
  static constexpr uint32_t kTmemCols = NR <= 32 ? 32 : NR <= 64 ? 64 : NR <= 128 ? 128 : 256;
  static constexpr size_t kSmem = (size_t)kStages * kStage + 256 + 1024;  // + barriers, flags, alignment
  static_assert(kStages >= 2, "two stages at least");
};

// out[split][m][n] = sum_{k in split} P[m, k] R[n, k]   (rows m < M, n < nr; FP32)
template <int NR>
__global__ void __launch_bounds__(kGThreads, 2)
bf16_gemm_nt_kernel(const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmR, int64_t M,
                    int nr, int64_t K, int64_t k_per_split, float* __restrict__ out, int64_t ldo,
                    int64_t split_stride) {
  using C = GemmCfg<NR>;
  constexpr int S = C::kStages;
  extern __shared__ uint8_t gsm_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(gsm_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * C::kStage);
  uint64_t* empty = full + S;
  uint64_t* done = empty + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  int* loads_issued = reinterpret_cast<int*>(tmem_slot + 2);    // K steps loaded
  int* loads_consumed = reinterpret_cast<int*>(tmem_slot + 3);  // K steps handed to the MMA
  int* mma_committed = reinterpret_cast<int*>(tmem_slot + 4);   // `done` committed
  const uint32_t polls = g_gemm_poll_limit;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kGM;
  const int64_t kb = (int64_t)blockIdx.y * k_per_split;
  const int64_t ke = (kb + k_per_split) < K ? (kb + k_per_split) : K;
  const int nk = ke > kb ? (int)((ke - kb + kGK - 1) / kGK) : 0;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *loads_issued = *loads_consumed = *mma_committed = 0;
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

  if (nk > 0 && warp == 0 && lane == 0) {
    // producer
    for (int t = 0; t < nk; ++t) {
      const int s = t % S;
      if (t >= S && !role_wait(&empty[s], (uint32_t)(((t / S) - 1) & 1), abort_flag, polls)) break;
      mbar_arrive_expect_tx(&full[s], C::kStage);
      const int x = (int)(kb + (int64_t)t * kGK);
      tma_load_2d(sbase + s * C::kStage, &tmP, x, (int)m0, &full[s]);
      tma_load_2d(sbase + s * C::kStage + C::kA, &tmR, x, 0, &full[s]);
      *loads_issued = t + 1;
    }
  } else if (nk > 0 && warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = umma_idesc(kGM, NR);
    int t = 0;
    for (; t < nk; ++t) {
      const int s = t % S;
      if (!role_wait(&full[s], (uint32_t)((t / S) & 1), abort_flag, polls)) break;
      *loads_consumed = t + 1;
      tc_fence_after();
      const uint32_t a = sbase + s * C::kStage, b = a + C::kA;
#pragma unroll
      for (int kk = 0; kk < kGK / 16; ++kk)
        tc_mma(tmem, umma_desc_sw128(a + kk * 32), umma_desc_sw128(b + kk * 32), idesc, (t > 0 || kk > 0) ? 1u : 0u);
      tc_commit(&empty[s]);
    }
    tc_commit(done);  // arrives when every MMA issued above has completed
    *mma_committed = 1;
  }
  bool ok = true;
  if (nk > 0) ok = role_wait(done, 0u, abort_flag, polls) && !*abort_flag;
  ok = __syncthreads_and(ok);  // every role has left its loop: nothing more is issued
  if (!ok && tid == 0) {
    // Work issued before the give-up still runs: wait (bounded) for the TMA loads the MMA
    // issuer did not consume (each stage holds at most one such load, so its parity is
    // unambiguous) and for the committed MMAs, before shared memory and TMEM are released.
    for (int t = *loads_consumed; t < *loads_issued; ++t)
      mbar_wait_bounded(&full[t % S], (uint32_t)((t / S) & 1), kGemmDrainPolls);
    if (*mma_committed) mbar_wait_bounded(done, 0u, kGemmDrainPolls);
  }
  __syncthreads();
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
                                   int64_t ldqs, float* __restrict__ f_out, int64_t ldfo, int use_floor, float floor_v) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)np * nb;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / nb);
    const int64_t b = t % nb;
    __nv_bfloat16 hi = __float2bfloat16_rn(0.f), lo = hi;
    if (n < n_inst) {
      float f = F[b * ldf + n] + F[b * ldf + np + n];
      if (use_floor) f = fmaxf(f, floor_v);  // clamp_min of recon_osem_local_cntstat.py:7
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

// Joint batched EM update: w = a * (W[v][n] + W[v][np + n]) + b * wb[n][v] (wb may be NULL);
// plain: x * w / s; safe (recon_osem_plane_sparse.py:60-66): nan/inf -> 0 in w and s, then
// s > eps ? x * max(w, 0) / s : 0. s is per instance (lds > 0) or shared (lds = 0). Every
// operation is rounded separately, as jscc_em_update does; the next hi / lo pair into xs.
__global__ void batch_em_joint_kernel(const float* __restrict__ W, int64_t ldw, int64_t V, int n_inst, int np,
                                      float a, const float* __restrict__ wb, int64_t ldwb, float b,
                                      float* __restrict__ x, int64_t ldx, const float* __restrict__ s, int64_t lds,
                                      int safe, float eps, __nv_bfloat16* __restrict__ xs, int64_t ldxs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n_inst * V;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(t / V);
    const int64_t v = t % V;
    float w = __fmul_rn(a, __fadd_rn(W[v * ldw + n], W[v * ldw + np + n]));
    if (wb) w = __fadd_rn(w, __fmul_rn(b, wb[(int64_t)n * ldwb + v]));
    float sv = s[(int64_t)n * lds + v];
    float* px = x + (int64_t)n * ldx + v;
    float xn;
    if (!safe) {
      xn = __fdiv_rn(__fmul_rn(*px, w), sv);
    } else {
      w = isfinite(w) ? w : 0.f;
      sv = isfinite(sv) ? sv : 0.f;
      xn = sv > eps ? __fdiv_rn(__fmul_rn(*px, fmaxf(w, 0.f)), sv) : 0.f;
    }
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

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Tensor map of a row-major [rows x K] BF16 matrix (row stride ld elements), box = 64 K
// elements (128 bytes) x box_rows rows, 128-byte swizzle, zero fill outside the matrix.
bool make_map(CUtensorMap* map, const void* base, int64_t K, int64_t rows, int64_t ld, uint32_t box_rows) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)(K > 0 ? K : 8), (cuuint64_t)(rows > 0 ? rows : 1)};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kGK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NR>
int launch_gemm(const __nv_bfloat16* P, int64_t ldp, const __nv_bfloat16* R, int64_t ldr, int64_t M, int nr, int64_t K,
                int splits, float* out, int64_t ldo, float* part, cudaStream_t st) {
  using C = GemmCfg<NR>;
  // the shared-memory attribute is set once per device (outside any later graph capture: the
  // first call on a device happens eagerly)
  static std::atomic<unsigned long long> attr_set{0};
  int dev = 0;
  JSCC_CUDA_CHECK(cudaGetDevice(&dev));
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(attr_set.load() & bit)) {
    JSCC_CUDA_CHECK(cudaFuncSetAttribute(bf16_gemm_nt_kernel<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)C::kSmem));
    attr_set.fetch_or(bit);
  }
  int64_t kps = (K + splits - 1) / splits;
  kps = (kps + kGK - 1) / kGK * kGK;
  if (kps < kGK) kps = kGK;  // K = 0: one split whose tiles write zeros
  int64_t used = (K + kps - 1) / kps;
  if (used < 1) used = 1;
  CUtensorMap mp, mr;
  if (K > 0) {
    JSCC_REQUIRE(make_map(&mp, P, K, M, ldp, kGM) && make_map(&mr, R, K, nr, ldr, NR),
                 "jscc_bf16_gemm_nt: tensor map encoding failed");
  } else {
    memset(&mp, 0, sizeof(mp));
    memset(&mr, 0, sizeof(mr));
  }
  dim3 grid((unsigned)((M + kGM - 1) / kGM), (unsigned)used);
  float* dst = used > 1 ? part : out;
  const int64_t ldd = used > 1 ? nr : ldo;
  const int64_t sstride = used > 1 ? M * nr : 0;
  JSCC_TIMED("bf16_gemm_nt", st,
             (bf16_gemm_nt_kernel<NR><<<grid, kGThreads, C::kSmem, st>>>(mp, mr, M, nr, K, kps, dst, ldd, sstride)));
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
                     int32_t np, void* qs, int64_t ldqs, float* f_out, int64_t ldfo, int32_t use_floor, float floor_v,
                     void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && nb >= 0 && b0 >= 0, "jscc_batch_ratio: bad sizes");
  if (np == 0 || nb == 0) return JSCC_OK;
  JSCC_REQUIRE(F && y && qs, "jscc_batch_ratio: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_ratio", st,
             (batch_ratio_kernel<<<(unsigned)grid_blocks((int64_t)np * nb), 256, 0, st>>>(
                 F, ldf, y, ldy, b0, nb, n_inst, np, static_cast<__nv_bfloat16*>(qs), ldqs, f_out, ldfo, use_floor,
                 floor_v)));
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

int jscc_batch_em_joint(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np, float coef_a,
                        const float* w_b, int64_t ldwb, float coef_b, float* x, int64_t ldx, const float* s_map,
                        int64_t lds, int32_t mode, float eps, void* xs, int64_t ldxs, void* stream) {
  JSCC_REQUIRE(n_inst >= 0 && np >= n_inst && V >= 0 && lds >= 0, "jscc_batch_em_joint: bad sizes");
  JSCC_REQUIRE(mode == JSCC_EM_PLAIN || mode == JSCC_EM_SAFE, "jscc_batch_em_joint: bad mode %d", mode);
  if (n_inst == 0 || V == 0) return JSCC_OK;
  JSCC_REQUIRE(W && x && s_map, "jscc_batch_em_joint: null pointer argument");
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("batch_em", st,
             (batch_em_joint_kernel<<<(unsigned)grid_blocks((int64_t)n_inst * V), 256, 0, st>>>(
                 W, ldw, V, n_inst, np, coef_a, w_b, ldwb, coef_b, x, ldx, s_map, lds, mode == JSCC_EM_SAFE ? 1 : 0,
                 eps, static_cast<__nv_bfloat16*>(xs), ldxs)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

}  // extern "C"

namespace jscc {
// Poll bound of the GEMM's role waits on the current device (`reset` restores the default).
int set_gemm_poll_limit(uint32_t polls, bool reset) {
  const uint32_t v = reset ? kGemmPolls : polls;
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_gemm_poll_limit, &v, sizeof(v)));
  return JSCC_OK;
}
}  // namespace jscc

extern "C" {

int jscc_take_gemm_timeout_count(unsigned int* out) {
  JSCC_REQUIRE(out, "jscc_take_gemm_timeout_count: null pointer argument");
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_gemm_timeout_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_gemm_timeout_count, &zero, sizeof(zero)));
  *out = h;
  return JSCC_OK;
}

}  // extern "C"
