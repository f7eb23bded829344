// Shared device/host helpers for the JSCC OSEM kernels (sm_103a).
//
// Error model: every extern "C" entry point returns a jscc status code and
// leaves a human-readable message in a thread-local buffer that
// jscc_last_error() returns. No entry point allocates device memory: callers
// pass outputs and a workspace sized by the matching *_workspace_bytes call.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stddef.h>
#include <atomic>
#include <cstdio>
#include <cstdarg>

#include "../../include/jscc_gb300.h"

namespace jscc {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
std::atomic<unsigned long long>& launch_counter();

#define JSCC_REQUIRE(cond, ...)                                   \
  do {                                                            \
    if (!(cond)) {                                                \
      ::jscc::set_error(__VA_ARGS__);                             \
      return JSCC_ERR_INVALID;                                    \
    }                                                             \
  } while (0)

#define JSCC_CUDA_CHECK(expr)                                                  \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess) {                                                   \
      ::jscc::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                        __FILE__, __LINE__);                                   \
      return JSCC_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

// Checks the launch just issued and counts it.
#define JSCC_LAUNCH_CHECK()                                   \
  do {                                                        \
    ::jscc::launch_counter().fetch_add(1);                    \
    JSCC_CUDA_CHECK(cudaGetLastError());                      \
  } while (0)

// Optional per-kernel timing with CUDA events recorded on the launch stream
// (off by default; enabled by jscc_kernel_timing_enable for measurement runs,
// never while a stream is being captured into a graph).
bool timing_enabled();
void timing_begin(cudaStream_t st);
void timing_end(const char* name, cudaStream_t st);

#define JSCC_TIMED(name, st, ...)                      \
  do {                                                 \
    const bool _t = ::jscc::timing_enabled();          \
    if (_t) ::jscc::timing_begin(st);                  \
    __VA_ARGS__;                                       \
    if (_t) ::jscc::timing_end(name, st);              \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int num_sms();
// Read and clear the neighbour-table index counter of the prior kernel (prior.cu).
unsigned int take_prior_bad_index_count();

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carves aligned sub-buffers out of a caller-provided workspace.
struct Carver {
  char* base;
  size_t cap;
  size_t off = 0;
  Carver(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
  template <typename T>
  T* take(size_t count) {
    off = align_up(off, 256);
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
  bool ok() const { return off <= cap; }
};

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ float warp_sum(float v) {
  // Fixed xor-butterfly: the same lanes combine in the same order on every call.
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Streaming 128-bit load that does not pollute L1 (data read once per pass).
__device__ __forceinline__ float4 ld_stream_f4(const float* p) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}

__device__ __forceinline__ uint4 ld_stream_u4(const void* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

// ---------------------------------------------------------------- TMA bulk copies + mbarriers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later async-proxy
// (bulk copy) accesses of the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// One bulk global -> shared copy of `bytes` (multiple of 16; both addresses 16-byte
// aligned) completing on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Non-blocking test of phase `parity` of `bar` (never suspends the thread; for polling
// several barriers in turn).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`: false after max_polls unsuccessful polls
// (each poll may suspend briefly in hardware), so a lost copy cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Element loaders used by the generic (unaligned / tail) paths.
__device__ __forceinline__ float load_elem(const float* p, int64_t i) { return __ldg(p + i); }
__device__ __forceinline__ float load_elem(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

// ---------------------------------------------------------------- pipeline roles
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// named barrier `id` over `count` threads (the warps of one role)
__device__ __forceinline__ void role_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// named barrier returning the OR of every participant's `v` (the same value in all of them,
// so a decision taken on it is uniform within the role)
__device__ __forceinline__ bool role_sync_or(int id, int count, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

// bounded wait that also gives up once another thread has flagged an abort
__device__ __forceinline__ bool bk_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, uint32_t polls) {
  for (uint32_t i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 31u) == 31u && *abort_flag) return false;
  }
  return false;
}

// ------------------------------------------------------------------ cluster primitives
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t n_clusters_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// all threads of every CTA of the cluster
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// the address of this CTA's shared variable at `p` in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_to_rank(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
// 16 bytes into another CTA's shared memory, completing 16 transaction bytes on that CTA's
// mbarrier (no fence: the receiver's wait on its own mbarrier sees the data)
__device__ __forceinline__ void st_async_v4(uint32_t addr, float a, float b, float c, float d, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                   addr),
               "f"(a), "f"(b), "f"(c), "f"(d), "r"(bar)
               : "memory");
}
// a wait that sees arrivals (and the stores before them) from other CTAs of the cluster
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool cf_wait_cluster(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                                uint32_t polls) {
  for (uint32_t i = 0; i < polls; ++i) {
    if (mbar_try_wait_cluster(bar, parity)) return true;
    if ((i & 31u) == 31u && *abort_flag) return false;
  }
  return false;
}

}  // namespace jscc
