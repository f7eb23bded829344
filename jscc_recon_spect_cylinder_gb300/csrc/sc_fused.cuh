// Fused SC weight: forward projection, ratio and back-projection in one read of the rows.
//
// For one rotation of the image read directly (no gather, no inverse rotation),
// w += scale * A^T (proj / max(A x, floor)) over the bins b of one call
// (get_weight_single, recon_osem_plane.py:28-30). The two-pass form reads every row twice
// (forward, then back); here each row is read once:
//   * a cluster of two CTAs (one per SM) takes a contiguous range of the call's rows; CTA h
//     owns the columns [h * split, split) or [split, V) and keeps, per consumer thread, its
//     columns' image values and back-projection sums in registers (c = 4 t + 1,920 u);
//   * a producer warp streams every row's column half into a ring of shared-memory stages
//     (cp.async.bulk on mbarriers);
//   * per batch of up to `batch` rows (a body compiled per row count) the consumers form their
//     partial dots, reduce them per warp and then over the warps in warp order after one
//     named barrier, exchange the CTA's partials with the peer CTA (one 16-byte st.async
//     completing on the peer's mbarrier), and form f = partial(rank 0) + partial(rank 1) (the
//     same sum, so the same ratio, in both CTAs), r = proj / max(f, floor), then add r * row
//     to their sums, rows in order;
//   * every cluster writes one partial image; sc_reduce_scatter_kernel adds the clusters'
//     images in cluster order (scaled) to the weight.
// Every wait is bounded (jscc_set_wait_limit): a CTA that gives up counts it
// (jscc_take_wait_timeout_count), waits (bounded) for what it still has in flight and leaves
// through the final cluster barrier with its peer.
#pragma once

#include <type_traits>

namespace jscc {

constexpr int kFsThreads = 512;
constexpr int kFsConsumerWarps = 15;
constexpr int kFsConsumers = kFsConsumerWarps * 32;
constexpr int kFsProducerWarp = kFsConsumerWarps;
constexpr int kFsQ = 10;  // chunks of four columns per consumer thread: a half holds <= 19,200 columns
constexpr int kFsHalfMax = kFsQ * 4 * kFsConsumers;
constexpr int kFsMaxStages = 8;
constexpr int kFsMaxBatch = 4;  // rows per exchange (one 16-byte store)
constexpr int kFsHeader = 1024;
constexpr uint32_t kFsMaxPolls = 1u << 22;
constexpr uint32_t kFsDrainPolls = 1u << 20;
static_assert(kFsProducerWarp * 32 + 32 == kFsThreads, "warp roles");

__device__ unsigned int g_sc_timeout_count = 0;
__device__ uint32_t g_sc_poll_limit = kFsMaxPolls;

template <typename T>
struct FsRow;
template <>
struct FsRow<__nv_bfloat16> {
  // four consecutive row values from shared memory (c a multiple of 4)
  __device__ __forceinline__ static void get(const __nv_bfloat16* p, int c, float (&v)[4]) {
    const uint2 u = *reinterpret_cast<const uint2*>(p + c);
    v[0] = bf16_lo(u.x); v[1] = bf16_hi(u.x); v[2] = bf16_lo(u.y); v[3] = bf16_hi(u.y);
  }
};
template <>
struct FsRow<float> {
  __device__ __forceinline__ static void get(const float* p, int c, float (&v)[4]) {
    const float4 u = *reinterpret_cast<const float4*>(p + c);
    v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
  }
};

template <typename T>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kFsThreads, 1)
sc_fused_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx, int64_t n_bins,
                int64_t V, int64_t split, const float* __restrict__ x, const float* __restrict__ proj,
                int64_t ld_proj, int r0, int use_floor, float floor_v, float* __restrict__ part, int64_t ldp,
                int n_stages, int batch, uint32_t stage_stride) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kFsMaxStages]
  uint64_t* empty = full + kFsMaxStages;                // [kFsMaxStages]
  uint64_t* xfull = empty + kFsMaxStages;               // [2] the peer's partials, by batch parity
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 144);
  int* issued = reinterpret_cast<int*>(smem + 148);
  int* used = reinterpret_cast<int*>(smem + 152);
  int* armed = reinterpret_cast<int*>(smem + 160);   // [2] phases of xfull armed
  int* waited = reinterpret_cast<int*>(smem + 168);  // [2] phases of xfull waited for by warp 0
  float* red = reinterpret_cast<float*>(smem + 256);   // [2][kFsConsumerWarps][kFsMaxBatch]
  float* xbuf = reinterpret_cast<float*>(smem + 768);  // [2][kFsMaxBatch] the peer's partials
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t h = cluster_rank();
  const int64_t cl = blockIdx.x >> 1, n_cl = gridDim.x >> 1;
  const int64_t rpc = (n_bins + n_cl - 1) / n_cl;
  const int64_t b0 = cl * rpc, b1 = b0 + rpc < n_bins ? b0 + rpc : n_bins;
  const int n_rows = b1 > b0 ? (int)(b1 - b0) : 0;
  const int64_t col0 = h == 0 ? 0 : split;
  const int ncol = (int)(h == 0 ? split : V - split);
  const uint32_t row_bytes = (uint32_t)ncol * (uint32_t)sizeof(T);
  const uint32_t polls = g_sc_poll_limit;
  auto stage = [&](int s) { return reinterpret_cast<const T*>(smem + kFsHeader + (size_t)s * stage_stride); };
  if (tid == 0) {
    for (int s = 0; s < kFsMaxStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, kFsConsumerWarps);
    }
    mbar_init(xfull, 1);
    mbar_init(xfull + 1, 1);
    *abort_flag = 0;
    *issued = *used = 0;
    armed[0] = armed[1] = waited[0] = waited[1] = 0;
    mbar_init_fence();
  }
  __syncthreads();
  cluster_sync_all();  // the peer's barriers are initialised before any exchange
  if (warp == kFsProducerWarp) {
    // ---------------------------------------------------------------- producer warp
    int win_base = INT_MIN;
    int64_t win_val = 0;  // 32 row indices of the window, one per lane
    bool ok = true;
    for (int k = 0; k < n_rows && ok; ++k) {
      const int s = k % n_stages;
      if (k >= n_stages) {
        bool w = lane == 0 ? bk_wait(empty + s, (uint32_t)(k / n_stages - 1) & 1u, abort_flag, polls) : true;
        ok = __shfl_sync(0xffffffffu, w, 0);
        if (!ok) break;
      }
      if (win_base == INT_MIN || k >= win_base + 32) {
        win_base = k;
        win_val = k + lane < n_rows ? (row_idx ? row_idx[b0 + k + lane] : b0 + k + lane) : 0;
      }
      const int64_t pb = __shfl_sync(0xffffffffu, win_val, k - win_base);
      if (lane == 0) {
        mbar_arrive_expect_tx(full + s, row_bytes);
        bulk_copy_g2s(const_cast<T*>(stage(s)), A + pb * lda + col0, row_bytes, full + s);
        *issued = k + 1;
      }
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else {
    // ---------------------------------------------------------------- consumer warps
    float4 xv[kFsQ], acc[kFsQ];
#pragma unroll
    for (int u = 0; u < kFsQ; ++u) {
      const int c = tid * 4 + u * (kFsConsumers * 4);
      xv[u] = c < ncol ? *reinterpret_cast<const float4*>(x + col0 + c) : make_float4(0.f, 0.f, 0.f, 0.f);
      acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    bool bad = false, aborted = false;
    int par = 0, i = 0;
    // One batch of NB rows from row bs; false when a wait gave up. The body is compiled once
    // per row count, so a batch issues no instructions for rows it does not hold.
    auto run_batch = [&](auto nb_tag, int bs) -> bool {
      constexpr int NB = decltype(nb_tag)::value;
      // this lane's row of the batch: its projection value, read before the dots
      float y_lane = 0.f;
      if (lane < NB) {
        const int64_t b = b0 + bs + lane;
        const int64_t pb = row_idx ? row_idx[b] : b;
        y_lane = proj[pb * ld_proj + r0];
      }
      int sl[NB];
#pragma unroll
      for (int k = 0; k < NB; ++k) sl[k] = (bs + k) % n_stages;
#pragma unroll
      for (int k = 0; k < NB; ++k)
        if (!bk_wait(full + sl[k], (uint32_t)((bs + k) / n_stages) & 1u, abort_flag, polls)) bad = true;
      // ---- partial dots over this CTA's columns
      float4 pd[NB];
#pragma unroll
      for (int k = 0; k < NB; ++k) pd[k] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < kFsQ; ++u) {
        const int c = tid * 4 + u * (kFsConsumers * 4);
        if (c < ncol) {
#pragma unroll
          for (int k = 0; k < NB; ++k) {
            float v[4];
            FsRow<T>::get(stage(sl[k]), c, v);
            const float2 lo = __ffma2_rn(make_float2(v[0], v[1]), make_float2(xv[u].x, xv[u].y),
                                         make_float2(pd[k].x, pd[k].y));
            const float2 hi = __ffma2_rn(make_float2(v[2], v[3]), make_float2(xv[u].z, xv[u].w),
                                         make_float2(pd[k].z, pd[k].w));
            pd[k] = make_float4(lo.x, lo.y, hi.x, hi.y);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        const float f = warp_sum((pd[k].x + pd[k].y) + (pd[k].z + pd[k].w));
        if (lane == 0) red[(par * kFsConsumerWarps + warp) * kFsMaxBatch + k] = f;
      }
      if (role_sync_or(1, kFsConsumers, bad)) return false;
      // ---- this CTA's partial of row k in lane k (warps in order), to the peer
      float mine = 0.f;
      if (lane < NB)
        for (int w = 0; w < kFsConsumerWarps; ++w) mine += red[(par * kFsConsumerWarps + w) * kFsMaxBatch + lane];
      if (warp == 0) {
        const float m0 = __shfl_sync(0xffffffffu, mine, 0), m1 = __shfl_sync(0xffffffffu, mine, 1);
        const float m2 = __shfl_sync(0xffffffffu, mine, 2), m3 = __shfl_sync(0xffffffffu, mine, 3);
        if (lane == 0) {
          mbar_arrive_expect_tx(xfull + par, 16);  // the peer's 16 bytes for this batch
          armed[par] += 1;
          const uint32_t peer = h ^ 1u;
          st_async_v4(map_to_rank(xbuf + par * kFsMaxBatch, peer), m0, m1, m2, m3, map_to_rank(xfull + par, peer));
        }
      }
      // ---- the peer's partials; f = partial(rank 0) + partial(rank 1) in both CTAs
      const bool got = cf_wait_cluster(xfull + par, (uint32_t)(i >> 1) & 1u, abort_flag, polls);
      if (warp == 0 && lane == 0 && got) waited[par] += 1;
      if (!__all_sync(0xffffffffu, got)) return false;
      float r_lane = 0.f;
      if (lane < NB) {
        const float theirs = xbuf[par * kFsMaxBatch + lane];
        float f = h == 0 ? mine + theirs : theirs + mine;
        if (use_floor) f = fmaxf(f, floor_v);
        r_lane = y_lane / f;
      }
      // ---- back-projection: acc += r_k * row_k over this thread's columns, rows in order
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        const float rk = __shfl_sync(0xffffffffu, r_lane, k);
#pragma unroll
        for (int u = 0; u < kFsQ; ++u) {
          const int c = tid * 4 + u * (kFsConsumers * 4);
          if (c < ncol) {
            float v[4];
            FsRow<T>::get(stage(sl[k]), c, v);
            const float2 rr = make_float2(rk, rk);
            const float2 lo = __ffma2_rn(rr, make_float2(v[0], v[1]), make_float2(acc[u].x, acc[u].y));
            const float2 hi = __ffma2_rn(rr, make_float2(v[2], v[3]), make_float2(acc[u].z, acc[u].w));
            acc[u] = make_float4(lo.x, lo.y, hi.x, hi.y);
          }
        }
      }
      // ---- this warp is past its reads of the batch's stages
      __syncwarp();
      if (lane == 0) {
        if (warp == 0) *used = bs + NB;
#pragma unroll
        for (int k = 0; k < NB; ++k) mbar_arrive(empty + sl[k]);
      }
      return true;
    };
    for (int bs = 0; bs < n_rows; bs += batch, par ^= 1, ++i) {
      const int n = n_rows - bs < batch ? n_rows - bs : batch;
      bool ok;
      if (n == 1) {
        ok = run_batch(std::integral_constant<int, 1>{}, bs);
      } else if (n == 2) {
        ok = run_batch(std::integral_constant<int, 2>{}, bs);
      } else if (n == 3) {
        ok = run_batch(std::integral_constant<int, 3>{}, bs);
      } else {
        ok = run_batch(std::integral_constant<int, kFsMaxBatch>{}, bs);
      }
      if (!ok) {
        aborted = true;
        break;
      }
    }
    if (aborted) {
      *abort_flag = 1;
    } else {
      float* out = part + cl * ldp + col0;
#pragma unroll
      for (int u = 0; u < kFsQ; ++u) {
        const int c = tid * 4 + u * (kFsConsumers * 4);
        if (c < ncol) *reinterpret_cast<float4*>(out + c) = acc[u];
      }
    }
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_sc_timeout_count, 1u);
    // copies still in flight write this CTA's shared memory: wait (bounded) for them
    const int last = *issued;
    for (int k = *used > last - n_stages ? *used : (last - n_stages > 0 ? last - n_stages : 0); k < last; ++k)
      mbar_wait_bounded(full + k % n_stages, (uint32_t)(k / n_stages) & 1u, kFsDrainPolls);
    for (int p = 0; p < 2; ++p)  // a peer store this CTA armed for and did not see land
      if (armed[p] > waited[p]) mbar_wait_bounded(xfull + p, (uint32_t)(armed[p] - 1) & 1u, kFsDrainPolls);
  }
  __syncthreads();
  cluster_sync_all();  // no CTA leaves while its peer may still write its shared memory
}

}  // namespace jscc
