// Single-photon (self-collimation, SC) projector: w += scale * sum_r P_r^-1 A^T (y_r / A P_r x).
//
// Reference semantics: recon_osem_plane.py:28-30 (get_weight_single) inside the
// rotation loop of osem_bin_mode (recon_osem_plane.py:49-53); the clamped form of
// recon_osem_local_cntstat.py:6-8.
//
// GB300 design
//  * All rotations of one call share the subset matrix A, so the R rotated images
//    are gathered once into X[R][V] and A is streamed once per pass for up to 8
//    rotations (a skinny GEMM instead of R GEMVs).
//  * Forward pass: CTA per row block, 128-bit streaming loads of A that bypass L1,
//    X re-read from L1/L2, fixed-order CTA reduction, ratio epilogue fused.
//  * Back pass: CTA per (1024-column tile x row chunk); each thread owns 4 (fp32)
//    or 8 (bf16) adjacent columns and walks its rows in order; partial column sums
//    go to the workspace.
//  * Reduce pass: one thread per output voxel sums the chunk partials in chunk
//    order, applies the inverse rotation gather and accumulates into `weight`.
//  No float atomics anywhere: every sum has one fixed order, so results are
//  bit-reproducible run to run.
#include "jscc_common.cuh"

#include <mutex>

#include "sc_fused.cuh"

namespace jscc {

constexpr int kRotBlock = 8;          // rotations handled per pass over A
constexpr int kColTile = 1024;        // columns per back-pass CTA
constexpr int kTargetCtas = 1216;     // back-pass grid target (8 CTAs x 152 SMs)
constexpr int kFwdThreads = 256;

__device__ unsigned int g_bad_index_count = 0;  // out-of-range rotation indices seen

// ------------------------------------------------------------------ gather
__global__ void sc_gather_rot_kernel(const float* __restrict__ img, const int64_t* __restrict__ rotmat,
                                     int64_t ld_rot, int r0, int nr, int64_t V, int64_t ldx,
                                     float* __restrict__ xr) {
  const int64_t total = (int64_t)nr * V;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / V);
    const int64_t j = t - (int64_t)r * V;
    int64_t src = j;
    if (rotmat != nullptr) {
      src = rotmat[j * ld_rot + r0 + r] - 1;
      if (src < 0 || src >= V) {
        atomicAdd(&g_bad_index_count, 1u);
        xr[(int64_t)r * ldx + j] = 0.f;
        continue;
      }
    }
    xr[(int64_t)r * ldx + j] = img[src];
  }
}

// ------------------------------------------------------------------ forward
template <typename T>
struct VecTraits;
template <>
struct VecTraits<float> {
  static constexpr int kVec = 4;  // elements per 16-byte load
};
template <>
struct VecTraits<__nv_bfloat16> {
  static constexpr int kVec = 8;
};

template <typename T>
__device__ __forceinline__ void load_vec(const T* p, float (&v)[VecTraits<T>::kVec]);

template <>
__device__ __forceinline__ void load_vec<float>(const float* p, float (&v)[4]) {
  float4 a = ld_stream_f4(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
template <>
__device__ __forceinline__ void load_vec<__nv_bfloat16>(const __nv_bfloat16* p, float (&v)[8]) {
  uint4 u = ld_stream_u4(p);
  v[0] = bf16_lo(u.x); v[1] = bf16_hi(u.x);
  v[2] = bf16_lo(u.y); v[3] = bf16_hi(u.y);
  v[4] = bf16_lo(u.z); v[5] = bf16_hi(u.z);
  v[6] = bf16_lo(u.w); v[7] = bf16_hi(u.w);
}

// acc + sum_k a[k] * x[k] over one 16-byte vector of A held as raw bits.
template <typename T>
__device__ __forceinline__ float fma_raw(const uint4& u, const float* x, float acc);
template <>
__device__ __forceinline__ float fma_raw<float>(const uint4& u, const float* x, float acc) {
  const float4 xv = *reinterpret_cast<const float4*>(x);
  acc = fmaf(__uint_as_float(u.x), xv.x, acc);
  acc = fmaf(__uint_as_float(u.y), xv.y, acc);
  acc = fmaf(__uint_as_float(u.z), xv.z, acc);
  acc = fmaf(__uint_as_float(u.w), xv.w, acc);
  return acc;
}
template <>
__device__ __forceinline__ float fma_raw<__nv_bfloat16>(const uint4& u, const float* x, float acc) {
  const float4 x0 = *reinterpret_cast<const float4*>(x);
  const float4 x1 = *reinterpret_cast<const float4*>(x + 4);
  acc = fmaf(bf16_lo(u.x), x0.x, acc);
  acc = fmaf(bf16_hi(u.x), x0.y, acc);
  acc = fmaf(bf16_lo(u.y), x0.z, acc);
  acc = fmaf(bf16_hi(u.y), x0.w, acc);
  acc = fmaf(bf16_lo(u.z), x1.x, acc);
  acc = fmaf(bf16_hi(u.z), x1.y, acc);
  acc = fmaf(bf16_lo(u.w), x1.z, acc);
  acc = fmaf(bf16_hi(u.w), x1.w, acc);
  return acc;
}

// ratio[b][r] = proj[b, r0 + r] / f(b, r), f = A[b,:] . X[r,:]
template <typename T, int ROWS, int RB, bool VEC>
__global__ void __launch_bounds__(kFwdThreads)
sc_forward_ratio_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx,
                        int64_t n_bins, int64_t V, const float* __restrict__ xr, int64_t ldx, int nr,
                        const float* __restrict__ proj, int64_t ld_proj, int r0, int use_floor,
                        float floor_v, float* __restrict__ ratio) {
  constexpr int NV = VecTraits<T>::kVec;
  constexpr int NW = kFwdThreads / 32;
  __shared__ float red[NW][ROWS * RB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t nblk = (n_bins + ROWS - 1) / ROWS;

  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t b0 = blk * ROWS;
    float acc[ROWS][RB];
#pragma unroll
    for (int i = 0; i < ROWS; ++i)
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[i][r] = 0.f;

    const T* rowp[ROWS];
#pragma unroll
    for (int i = 0; i < ROWS; ++i) {
      int64_t b = b0 + i;
      const int64_t bb = b < n_bins ? b : n_bins - 1;  // clamped; masked below
      rowp[i] = A + (row_idx ? row_idx[bb] : bb) * lda;
    }

    int64_t tail_start = 0;
    if (VEC) {
      const int64_t nvec = V / NV;
      tail_start = nvec * NV;
#pragma unroll 2
      for (int64_t v = tid; v < nvec; v += kFwdThreads) {
        float a[ROWS][NV];
#pragma unroll
        for (int i = 0; i < ROWS; ++i) load_vec<T>(rowp[i] + v * NV, a[i]);
#pragma unroll
        for (int r = 0; r < RB; ++r) {
          if (r < nr) {
            const float* xp = xr + (int64_t)r * ldx + v * NV;
            float x[NV];
#pragma unroll
            for (int k = 0; k < NV; k += 4) {
              float4 q = __ldg(reinterpret_cast<const float4*>(xp + k));
              x[k] = q.x; x[k + 1] = q.y; x[k + 2] = q.z; x[k + 3] = q.w;
            }
#pragma unroll
            for (int i = 0; i < ROWS; ++i)
#pragma unroll
              for (int k = 0; k < NV; ++k) acc[i][r] = fmaf(a[i][k], x[k], acc[i][r]);
          }
        }
      }
    }
    for (int64_t j = tail_start + tid; j < V; j += kFwdThreads) {
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        if (r < nr) {
          const float x = __ldg(xr + (int64_t)r * ldx + j);
#pragma unroll
          for (int i = 0; i < ROWS; ++i) acc[i][r] = fmaf(load_elem(rowp[i], j), x, acc[i][r]);
        }
      }
    }

    // fixed-order CTA reduction
#pragma unroll
    for (int i = 0; i < ROWS; ++i)
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        float s = warp_sum(acc[i][r]);
        if (lane == 0) red[warp][i * RB + r] = s;
      }
    __syncthreads();
    if (tid < ROWS * RB) {
      const int i = tid / RB, r = tid % RB;
      const int64_t b = b0 + i;
      if (b < n_bins && r < nr) {
        float f = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) f += red[w][tid];
        if (use_floor) f = fmaxf(f, floor_v);
        const int64_t pb = row_idx ? row_idx[b] : b;
        ratio[b * RB + r] = proj[pb * ld_proj + r0 + r] / f;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ forward, balanced split
// The subset matrix is viewed as n_bins x nvr vector units (nvr = ceil(V / NV)). Every
// warp of the persistent grid owns one contiguous range of L units (the last warp
// fewer), so all warps stream the same number of bytes. A range crosses at most a
// few row boundaries; for each row piece the warp writes one partial dot product
// per rotation to part[g][k][RB]. sc_finish_ratio_kernel sums a row's partials in
// warp order. The rotated image(s) are staged in shared memory when they fit.
template <typename T, int RB, bool VEC, bool SMEM_X, int THREADS>
__global__ void __launch_bounds__(THREADS)
sc_forward_split_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx,
                        int64_t n_bins, int64_t V, const float* __restrict__ xr, int64_t ldx_src,
                        int64_t ldx, int nr, int64_t nvr, int64_t L, int maxp,
                        float* __restrict__ part) {
  constexpr int NV = VEC ? VecTraits<T>::kVec : 1;
  constexpr int WARPS = THREADS / 32;
  extern __shared__ float4 xs4[];
  float* xs = reinterpret_cast<float*>(xs4);
  const int lane = threadIdx.x & 31;
  const int64_t g = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
  if (SMEM_X) {
    for (int r = 0; r < nr; ++r)
      for (int64_t i = threadIdx.x; i < V; i += THREADS) xs[(int64_t)r * ldx + i] = __ldg(xr + r * ldx_src + i);
    __syncthreads();
  } else {
    ldx = ldx_src;
  }
  const float* xsrc = SMEM_X ? xs : xr;
  const int64_t U = n_bins * nvr;
  int64_t u = g * L;
  const int64_t u_end = (u + L < U) ? u + L : U;
  int64_t row = u < U ? u / nvr : 0;
  int k = 0;
  while (u < u_end) {
    const int64_t row_end = (row + 1) * nvr;
    const int64_t piece_end = row_end < u_end ? row_end : u_end;
    const T* rowp = A + (row_idx ? row_idx[row] : row) * lda;
    const int64_t ubase = row * nvr;
    float acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = 0.f;
    int64_t uu = u + lane;
    if constexpr (VEC) {
      // 4 independent 16-byte loads in flight per lane; raw registers, converted on use.
      // Only whole vectors here (32-bit column arithmetic); the row's partial last
      // vector, if any, is left to the loop below.
      const int64_t full_end_u = ubase + V / NV;
      const int64_t fe = piece_end < full_end_u ? piece_end : full_end_u;
      if (uu + 96 < fe) {
        const T* rp = rowp;
        const float* xp0 = xsrc;
        int col = (int)(uu - ubase) * NV;
        const int n_iter = (int)((fe - uu - 96 + 127) / 128);
        for (int it = 0; it < n_iter; ++it, col += 128 * NV) {
          uint4 raw[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) raw[q] = ld_stream_u4(rp + col + 32 * NV * q);
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int r = 0; r < RB; ++r)
              if (r < nr) acc[r] = fma_raw<T>(raw[q], xp0 + (int64_t)r * ldx + col + 32 * NV * q, acc[r]);
        }
        uu += (int64_t)n_iter * 128;
      }
    }
    for (; uu < piece_end; uu += 32) {
      const int64_t col = (uu - ubase) * NV;
      bool done = false;
      if constexpr (VEC) {
        if (col + NV <= V) {
          float a[NV];
          load_vec<T>(rowp + col, a);
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            if (r < nr) {
              const float* xp = xsrc + (int64_t)r * ldx + col;
#pragma unroll
              for (int kk = 0; kk < NV; ++kk) acc[r] = fmaf(a[kk], xp[kk], acc[r]);
            }
          }
          done = true;
        }
      }
      if (!done) {
        const int64_t cend = (col + NV < V) ? col + NV : V;
        for (int64_t c = col; c < cend; ++c) {
          const float av = load_elem(rowp, c);
#pragma unroll
          for (int r = 0; r < RB; ++r)
            if (r < nr) acc[r] = fmaf(av, xsrc[(int64_t)r * ldx + c], acc[r]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      const float sum = warp_sum(acc[r]);
      if (lane == 0) part[((g * maxp) + k) * RB + r] = sum;
    }
    ++k;
    ++row;
    u = piece_end;
  }
}

// ratio[b][r] = proj[b, r0 + r] / f, f = sum of the row's partials in warp order.
template <int RB>
__global__ void sc_finish_ratio_kernel(const float* __restrict__ part, int64_t n_bins, int64_t nvr,
                                       int64_t L, int maxp, const int64_t* __restrict__ row_idx,
                                       const float* __restrict__ proj, int64_t ld_proj, int r0, int nr,
                                       int use_floor, float floor_v, float* __restrict__ ratio) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_bins * RB;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / RB;
    const int r = (int)(t % RB);
    if (r >= nr) continue;
    const int64_t g0 = (b * nvr) / L;
    const int64_t g1 = ((b + 1) * nvr - 1) / L;
    float f = 0.f;
    for (int64_t g = g0; g <= g1; ++g) {
      const int64_t first_row = (g * L) / nvr;
      f += part[((g * maxp) + (b - first_row)) * RB + r];
    }
    if (use_floor) f = fmaxf(f, floor_v);
    const int64_t pb = row_idx ? row_idx[b] : b;
    ratio[b * RB + r] = proj[pb * ld_proj + r0 + r] / f;
  }
}

// out[b][r0 + r] = f(b, r) (the forward projection itself, no ratio)
template <int RB>
__global__ void sc_finish_raw_kernel(const float* __restrict__ part, int64_t n_bins, int64_t nvr, int64_t L,
                                     int maxp, int r0, int nr, float* __restrict__ out, int64_t ld_out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_bins * RB;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / RB;
    const int r = (int)(t % RB);
    if (r >= nr) continue;
    const int64_t g0 = (b * nvr) / L;
    const int64_t g1 = ((b + 1) * nvr - 1) / L;
    float f = 0.f;
    for (int64_t g = g0; g <= g1; ++g) {
      const int64_t first_row = (g * L) / nvr;
      f += part[((g * maxp) + (b - first_row)) * RB + r];
    }
    out[b * ld_out + r0 + r] = f;
  }
}

// ratio[b][r] = g[b][r0 + r] (a caller-given vector to back-project)
template <int RB>
__global__ void sc_load_ratio_kernel(const float* __restrict__ g, int64_t ld_g, int64_t n_bins, int r0, int nr,
                                     float* __restrict__ ratio) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_bins * RB;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / RB;
    const int r = (int)(t % RB);
    ratio[t] = r < nr ? g[b * ld_g + r0 + r] : 0.f;
  }
}

// ------------------------------------------------------------------ back (partials)
// part[chunk][r][col] = sum_{b in chunk} A[b, col] * ratio[b][r]
template <typename T, int RB, bool VEC>
__global__ void __launch_bounds__(kColTile / VecTraits<T>::kVec)
sc_back_partial_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx,
                       int64_t n_bins, int64_t V,
                       const float* __restrict__ ratio, int nr, int64_t rows_per_chunk,
                       float* __restrict__ part, int64_t ldp) {
  constexpr int NV = VecTraits<T>::kVec;
  const int64_t col = (int64_t)blockIdx.x * kColTile + (int64_t)threadIdx.x * NV;
  const int64_t b_begin = (int64_t)blockIdx.y * rows_per_chunk;
  int64_t b_end = b_begin + rows_per_chunk;
  if (b_end > n_bins) b_end = n_bins;
  if (col >= V) return;
  const bool full = VEC && (col + NV <= V);

  float acc[RB][NV];
#pragma unroll
  for (int r = 0; r < RB; ++r)
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[r][k] = 0.f;

  if (full) {
    int64_t b = b_begin;
    for (; b + 4 <= b_end; b += 4) {
      float a[4][NV];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        load_vec<T>(A + (row_idx ? row_idx[b + u] : b + u) * lda + col, a[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int r = 0; r < RB; ++r) {
          if (r < nr) {
            const float q = __ldg(ratio + (b + u) * RB + r);
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[r][k] = fmaf(a[u][k], q, acc[r][k]);
          }
        }
      }
    }
    for (; b < b_end; ++b) {
      float a[NV];
      load_vec<T>(A + (row_idx ? row_idx[b] : b) * lda + col, a);
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        if (r < nr) {
          const float q = __ldg(ratio + b * RB + r);
#pragma unroll
          for (int k = 0; k < NV; ++k) acc[r][k] = fmaf(a[k], q, acc[r][k]);
        }
      }
    }
  } else {
    const int ncol = (int)((V - col) < NV ? (V - col) : NV);
    for (int64_t b = b_begin; b < b_end; ++b) {
      const T* rowb = A + (row_idx ? row_idx[b] : b) * lda;
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        if (r < nr) {
          const float q = __ldg(ratio + b * RB + r);
#pragma unroll
          for (int k = 0; k < NV; ++k)
            if (k < ncol) acc[r][k] = fmaf(load_elem(rowb, col + k), q, acc[r][k]);
        }
      }
    }
  }

  const int ncol = (int)((V - col) < NV ? (V - col) : NV);
#pragma unroll
  for (int r = 0; r < RB; ++r) {
    if (r < nr) {
      float* dst = part + ((int64_t)blockIdx.y * RB + r) * ldp + col;
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k < ncol) dst[k] = acc[r][k];
    }
  }
}

// ------------------------------------------------------------------ compensated column sums
// Kahan summation (Kahan 1965): s accumulates, c carries the rounding error of each add with
// the opposite sign; every add is an explicit round-to-nearest op so nothing is contracted.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// sum[chunk][col] / comp[chunk][col]: compensated column sums of the chunk's rows of A.
template <typename T, bool VEC>
__global__ void __launch_bounds__(kColTile / VecTraits<T>::kVec)
sc_colsum_kahan_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx, int64_t n_bins,
                       int64_t V, int64_t rows_per_chunk, float* __restrict__ sum, float* __restrict__ comp,
                       int64_t ldp) {
  constexpr int NV = VecTraits<T>::kVec;
  const int64_t col = (int64_t)blockIdx.x * kColTile + (int64_t)threadIdx.x * NV;
  const int64_t b_begin = (int64_t)blockIdx.y * rows_per_chunk;
  int64_t b_end = b_begin + rows_per_chunk;
  if (b_end > n_bins) b_end = n_bins;
  if (col >= V) return;
  const int ncol = (int)((V - col) < NV ? (V - col) : NV);
  float sa[NV], ca[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) sa[k] = ca[k] = 0.f;
  if (VEC && ncol == NV) {
    for (int64_t b = b_begin; b < b_end; ++b) {
      float a[NV];
      load_vec<T>(A + (row_idx ? row_idx[b] : b) * lda + col, a);
#pragma unroll
      for (int k = 0; k < NV; ++k) kahan_add(sa[k], ca[k], a[k]);
    }
  } else {
    for (int64_t b = b_begin; b < b_end; ++b) {
      const T* rowb = A + (row_idx ? row_idx[b] : b) * lda;
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k < ncol) kahan_add(sa[k], ca[k], load_elem(rowb, col + k));
    }
  }
  float* ds = sum + (int64_t)blockIdx.y * ldp + col;
  float* dc = comp + (int64_t)blockIdx.y * ldp + col;
#pragma unroll
  for (int k = 0; k < NV; ++k)
    if (k < ncol) {
      ds[k] = sa[k];
      dc[k] = ca[k];
    }
}

// ------------------------------------------------------------------ reduce + inverse rotation
__global__ void sc_reduce_scatter_kernel(const float* __restrict__ part, int64_t ldp, int chunks,
                                         int nr, int rb_stride, const int64_t* __restrict__ rotinv,
                                         int64_t ld_rot, int r0, int64_t V, int has_scale,
                                         float scale, float* __restrict__ weight) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V;
       j += (int64_t)gridDim.x * blockDim.x) {
    float acc = weight[j];
    for (int r = 0; r < nr; ++r) {
      int64_t src = j;
      if (rotinv != nullptr) {
        src = rotinv[j * ld_rot + r0 + r] - 1;
        if (src < 0 || src >= V) {
          atomicAdd(&g_bad_index_count, 1u);
          continue;
        }
      }
      float s = 0.f;
      for (int c = 0; c < chunks; ++c) s += part[((int64_t)c * rb_stride + r) * ldp + src];
      acc = has_scale ? __fadd_rn(acc, __fmul_rn(scale, s)) : __fadd_rn(acc, s);
    }
    weight[j] = acc;
  }
}

// SC sensitivity: s[j] += (sum_r colsum[rotinv[j, r] - 1]) / n_rot, colsum[c] = the chunk
// partials of column c and their carried errors summed in chunk order with compensation
// (rotations summed first, then divided, as main_local_cntstat.py:140-146 does).

__global__ void sc_sensitivity_kernel(const float* __restrict__ sum, const float* __restrict__ comp, int64_t ldp,
                                      int chunks, const int64_t* __restrict__ rotinv, int64_t ld_rot, int n_rot,
                                      int64_t V, float* __restrict__ weight) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V;
       j += (int64_t)gridDim.x * blockDim.x) {
    float acc = 0.f, acc_c = 0.f;
    for (int r = 0; r < n_rot; ++r) {
      int64_t src = j;
      if (rotinv != nullptr) {
        src = rotinv[j * ld_rot + r] - 1;
        if (src < 0 || src >= V) {
          atomicAdd(&g_bad_index_count, 1u);
          continue;
        }
      }
      // the chunk sums and their carried errors, compensated in chunk order
      float s = 0.f, c = 0.f;
      for (int k = 0; k < chunks; ++k) {
        kahan_add(s, c, sum[(int64_t)k * ldp + src]);
        kahan_add(s, c, -comp[(int64_t)k * ldp + src]);
      }
      kahan_add(acc, acc_c, __fsub_rn(s, c));
    }
    weight[j] = __fadd_rn(weight[j], __fdiv_rn(__fsub_rn(acc, acc_c), (float)n_rot));
  }
}

// ------------------------------------------------------------------ host planning
struct ScPlan {
  int rb;                  // rotation block (1, 2, 4, 8)
  int64_t ldx;             // padded voxel stride of X / partials
  int64_t col_tiles;       // back pass: 1024-column tiles
  int64_t chunks;          // back pass: row chunks
  int64_t rows_per_chunk;
  int64_t fwd_warps;       // forward pass: warps of the persistent grid (32 per SM)
  int fwd_maxp;            // forward pass: row pieces per warp (upper bound)
  size_t ws_bytes;         // the two-pass kernels' workspace (the minimum)
  int64_t fs_clusters;     // fused single-read path (one rotation): clusters of two CTAs
  size_t fs_bytes;         // its partial images, after the two-pass carve
};

static int pow2_block(int n_rot) {
  int rb = 1;
  while (rb < n_rot && rb < kRotBlock) rb <<= 1;
  return rb;
}

static ScPlan plan_sc(int64_t n_bins, int64_t V, int32_t n_rot) {
  ScPlan p{};
  p.rb = pow2_block(n_rot < 1 ? 1 : n_rot);
  p.ldx = (int64_t)align_up((size_t)(V > 0 ? V : 1), 8);
  p.col_tiles = (V + kColTile - 1) / kColTile;
  if (p.col_tiles < 1) p.col_tiles = 1;
  int64_t chunks = (kTargetCtas + p.col_tiles - 1) / p.col_tiles;
  int64_t max_chunks = (n_bins + 15) / 16;  // at least 16 rows per chunk
  if (max_chunks < 1) max_chunks = 1;
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks < 1) chunks = 1;
  p.rows_per_chunk = (n_bins + chunks - 1) / chunks;
  if (p.rows_per_chunk < 1) p.rows_per_chunk = 1;
  p.chunks = (n_bins + p.rows_per_chunk - 1) / p.rows_per_chunk;
  if (p.chunks < 1) p.chunks = 1;
  p.fwd_warps = (int64_t)num_sms() * 32;
  p.fwd_maxp = (int)((n_bins + p.fwd_warps - 1) / p.fwd_warps) + 2;
  size_t bytes = 0;
  bytes += align_up((size_t)p.fwd_warps * p.fwd_maxp * p.rb * sizeof(float), 256);  // fwd partials
  bytes += align_up((size_t)p.rb * p.ldx * sizeof(float), 256);                   // X
  bytes += align_up((size_t)(n_bins > 0 ? n_bins : 1) * p.rb * sizeof(float), 256);  // ratio
  bytes += align_up((size_t)p.chunks * p.rb * p.ldx * sizeof(float), 256);          // partials
  p.ws_bytes = bytes + 256;
  p.fs_clusters = n_rot == 1 ? (int64_t)num_sms() / 2 : 0;
  if (p.fs_clusters > n_bins) p.fs_clusters = n_bins;
  p.fs_bytes = p.fs_clusters > 0 ? align_up((size_t)p.fs_clusters * p.ldx * sizeof(float), 256) + 256 : 0;
  return p;
}

int set_sc_poll_limit(uint32_t polls, bool reset) {
  const uint32_t v = reset ? kFsMaxPolls : polls;
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_sc_poll_limit, &v, sizeof(v)));
  return JSCC_OK;
}

int take_sc_timeout_count(unsigned int* out) {
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_sc_timeout_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_sc_timeout_count, &zero, sizeof(zero)));
  *out = h;
  return JSCC_OK;
}

// The fused single-read path's partial images: after the two-pass carve `cv` when the
// workspace holds them, else nullptr (the two-pass kernels run).
static float* fused_partials(const ScPlan& p, Carver cv) {
  if (p.fs_bytes == 0) return nullptr;
  float* f = cv.take<float>((size_t)p.fs_clusters * p.ldx);
  return cv.ok() ? f : nullptr;
}

template <typename T, int RB>
static int launch_sc_block(const T* A, int64_t lda, const int64_t* row_idx, int64_t n_bins, int64_t V,
                           const float* proj,
                           int64_t ld_proj, int64_t ld_rot, int r0, int nr, const int64_t* rotinv,
                           int use_floor, float floor_v, int has_scale, float scale,
                           float* weight, const ScPlan& p, float* xr, float* ratio, float* part,
                           float* fpart, const float* xsrc_direct, cudaStream_t st, int stage = 0,
                           float* fout = nullptr, int64_t ld_fout = 0, const float* gin = nullptr,
                           int64_t ld_gin = 0, float* fs_part = nullptr) {
  // stage 0: forward, ratio, back (the weight); 1: forward only into fout; 2: back-project gin
  constexpr int NV = VecTraits<T>::kVec;
  const bool vec_ok = ((lda * (int64_t)sizeof(T)) % 16 == 0) &&
                      (reinterpret_cast<uintptr_t>(A) % 16 == 0);
  const int sms = num_sms();
  // fused single-read path: the weight of one rotation read directly, halves of 16-byte rows
  // that fit the consumer registers, at least two stages of a row half
  if (RB == 1 && stage == 0 && nr == 1 && xsrc_direct != nullptr && rotinv == nullptr && fs_part != nullptr &&
      vec_ok && V % (16 / (int64_t)sizeof(T)) == 0 && p.fs_clusters > 0) {
    const int64_t el = 16 / (int64_t)sizeof(T);
    const int64_t split = (V / 2 + el - 1) / el * el;
    const uint32_t stride = (uint32_t)align_up((size_t)split * sizeof(T), 128);
    int stages = (int)((227u * 1024u - kFsHeader) / stride);
    if (stages > kFsMaxStages) stages = kFsMaxStages;
    int batch = stages / 2 < kFsMaxBatch ? stages / 2 : kFsMaxBatch;
    if (split <= kFsHalfMax && V - split <= kFsHalfMax && V - split > 0 && stages >= 2 && batch >= 1 &&
        reinterpret_cast<uintptr_t>(xsrc_direct) % 16 == 0) {
      const size_t smem = kFsHeader + (size_t)stages * stride;
      JSCC_CUDA_CHECK(cudaFuncSetAttribute(sc_fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      JSCC_TIMED("sc_fused", st,
                 (sc_fused_kernel<T><<<(unsigned)(2 * p.fs_clusters), kFsThreads, smem, st>>>(
                     A, lda, row_idx, n_bins, V, split, xsrc_direct, proj, ld_proj, r0, use_floor, floor_v, fs_part,
                     p.ldx, stages, batch, stride)));
      JSCC_LAUNCH_CHECK();
      int64_t blocks = (V + 255) / 256;
      if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
      if (blocks < 1) blocks = 1;
      JSCC_TIMED("sc_reduce_scatter", st,
                 sc_reduce_scatter_kernel<<<(unsigned)blocks, 256, 0, st>>>(fs_part, p.ldx, (int)p.fs_clusters, 1, 1,
                                                                            nullptr, ld_rot, r0, V, has_scale, scale,
                                                                            weight));
      JSCC_LAUNCH_CHECK();
      return JSCC_OK;
    }
  }
  // forward: balanced contiguous split over warps, then fixed-order row finish
  if (stage == 2) {
    int64_t blocks = (n_bins * RB + 255) / 256;
    if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
    if (blocks < 1) blocks = 1;
    JSCC_TIMED("sc_load_ratio", st,
               sc_load_ratio_kernel<RB><<<(unsigned)blocks, 256, 0, st>>>(gin, ld_gin, n_bins, r0, nr, ratio));
    JSCC_LAUNCH_CHECK();
  } else {
    constexpr int NVv = VecTraits<T>::kVec;
    const int64_t nvr = vec_ok ? (V + NVv - 1) / NVv : V;
    const int64_t U = n_bins * nvr;
    const int64_t G = p.fwd_warps;
    const int64_t L = (U + G - 1) / G;
    const size_t xbytes = (size_t)nr * p.ldx * sizeof(float);
    // identity rotation: read the image directly (no gather pass)
    const bool direct = xsrc_direct != nullptr;
    const float* xsrc = direct ? xsrc_direct : xr;
    const int64_t xld = direct ? 0 : p.ldx;
    const bool smem_x = RB <= 2 && xbytes <= 200 * 1024;
    cudaError_t attr_err = cudaSuccess;
    if (RB <= 2) {
      const unsigned grid = (unsigned)(G / 32);
      const size_t sh = smem_x ? xbytes : 0;
      if (vec_ok && smem_x) {
        attr_err = cudaFuncSetAttribute(sc_forward_split_kernel<T, RB, true, true, 1024>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
        JSCC_TIMED("sc_forward_split", st,
                   sc_forward_split_kernel<T, RB, true, true, 1024><<<grid, 1024, sh, st>>>(
                       A, lda, row_idx, n_bins, V, xsrc, xld, p.ldx, nr, nvr, L, p.fwd_maxp, fpart));
      } else if (vec_ok) {
        JSCC_TIMED("sc_forward_split", st,
                   sc_forward_split_kernel<T, RB, true, false, 1024><<<grid, 1024, 0, st>>>(
                       A, lda, row_idx, n_bins, V, xsrc, xld, p.ldx, nr, nvr, L, p.fwd_maxp, fpart));
      } else {
        JSCC_TIMED("sc_forward_split", st,
                   sc_forward_split_kernel<T, RB, false, false, 1024><<<grid, 1024, 0, st>>>(
                       A, lda, row_idx, n_bins, V, xsrc, xld, p.ldx, nr, nvr, L, p.fwd_maxp, fpart));
      }
    } else {
      const unsigned grid = (unsigned)(G / 8);
      if (vec_ok)
        JSCC_TIMED("sc_forward_split", st,
                   sc_forward_split_kernel<T, RB, true, false, 256><<<grid, 256, 0, st>>>(
                       A, lda, row_idx, n_bins, V, xsrc, xld, p.ldx, nr, nvr, L, p.fwd_maxp, fpart));
      else
        JSCC_TIMED("sc_forward_split", st,
                   sc_forward_split_kernel<T, RB, false, false, 256><<<grid, 256, 0, st>>>(
                       A, lda, row_idx, n_bins, V, xsrc, xld, p.ldx, nr, nvr, L, p.fwd_maxp, fpart));
    }
    JSCC_CUDA_CHECK(attr_err);
    JSCC_LAUNCH_CHECK();
    int64_t blocks = (n_bins * RB + 255) / 256;
    if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
    if (blocks < 1) blocks = 1;
    if (stage == 1) {
      JSCC_TIMED("sc_finish_raw", st,
                 sc_finish_raw_kernel<RB><<<(unsigned)blocks, 256, 0, st>>>(fpart, n_bins, nvr, L, p.fwd_maxp, r0, nr,
                                                                            fout, ld_fout));
      JSCC_LAUNCH_CHECK();
      return JSCC_OK;
    }
    JSCC_TIMED("sc_finish_ratio", st,
               sc_finish_ratio_kernel<RB><<<(unsigned)blocks, 256, 0, st>>>(
                   fpart, n_bins, nvr, L, p.fwd_maxp, row_idx, proj, ld_proj, r0, nr, use_floor,
                   floor_v, ratio));
    JSCC_LAUNCH_CHECK();
  }
  {
    dim3 grid((unsigned)p.col_tiles, (unsigned)p.chunks);
    const int threads = kColTile / NV;
    JSCC_TIMED("sc_back_partial", st, {
      if (vec_ok)
        sc_back_partial_kernel<T, RB, true><<<grid, threads, 0, st>>>(
            A, lda, row_idx, n_bins, V, ratio, nr, p.rows_per_chunk, part, p.ldx);
      else
        sc_back_partial_kernel<T, RB, false><<<grid, threads, 0, st>>>(
            A, lda, row_idx, n_bins, V, ratio, nr, p.rows_per_chunk, part, p.ldx);
    });
    JSCC_LAUNCH_CHECK();
  }
  {
    int64_t blocks = (V + 255) / 256;
    if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
    if (blocks < 1) blocks = 1;
    JSCC_TIMED("sc_reduce_scatter", st,
               sc_reduce_scatter_kernel<<<(unsigned)blocks, 256, 0, st>>>(
                   part, p.ldx, (int)p.chunks, nr, RB, rotinv, ld_rot, r0, V, has_scale, scale,
                   weight));
    JSCC_LAUNCH_CHECK();
  }
  return JSCC_OK;
}

template <typename T>
static int sc_weight_typed(const T* A, int64_t lda, const int64_t* row_idx, int64_t n_bins, int64_t V,
                           const float* proj,
                           int64_t ld_proj, int n_rot, const float* img, const int64_t* rotmat,
                           const int64_t* rotinv, int64_t ld_rot, int use_floor, float floor_v, int has_scale,
                           float scale, float* weight, const ScPlan& p, float* xr, float* ratio,
                           float* part, float* fpart, cudaStream_t st, int stage = 0, float* fout = nullptr,
                           int64_t ld_fout = 0, const float* gin = nullptr, int64_t ld_gin = 0,
                           float* fs_part = nullptr) {
  const int sms = num_sms();
  for (int r0 = 0; r0 < n_rot; r0 += p.rb) {
    const int nr = (n_rot - r0) < p.rb ? (n_rot - r0) : p.rb;
    const float* direct = nullptr;
    if (stage == 2) {
      // back-projection only: no image
    } else if (rotmat == nullptr && nr == 1 && (reinterpret_cast<uintptr_t>(img) % 16 == 0)) {
      direct = img;
    } else {
      int64_t total = (int64_t)nr * V;
      int64_t blocks = (total + 255) / 256;
      if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
      if (blocks < 1) blocks = 1;
      JSCC_TIMED("sc_gather_rot", st,
                 sc_gather_rot_kernel<<<(unsigned)blocks, 256, 0, st>>>(img, rotmat, ld_rot, r0, nr,
                                                                        V, p.ldx, xr));
      JSCC_LAUNCH_CHECK();
    }
    int rc;
    switch (p.rb) {
      case 1:
        rc = launch_sc_block<T, 1>(A, lda, row_idx, n_bins, V, proj, ld_proj, ld_rot, r0, nr, rotinv,
                                   use_floor, floor_v, has_scale, scale, weight, p, xr, ratio, part,
                                   fpart, direct, st, stage, fout, ld_fout, gin, ld_gin, fs_part);
        break;
      case 2:
        rc = launch_sc_block<T, 2>(A, lda, row_idx, n_bins, V, proj, ld_proj, ld_rot, r0, nr, rotinv,
                                   use_floor, floor_v, has_scale, scale, weight, p, xr, ratio, part,
                                   fpart, direct, st, stage, fout, ld_fout, gin, ld_gin);
        break;
      case 4:
        rc = launch_sc_block<T, 4>(A, lda, row_idx, n_bins, V, proj, ld_proj, ld_rot, r0, nr, rotinv,
                                   use_floor, floor_v, has_scale, scale, weight, p, xr, ratio, part,
                                   fpart, direct, st, stage, fout, ld_fout, gin, ld_gin);
        break;
      default:
        rc = launch_sc_block<T, 8>(A, lda, row_idx, n_bins, V, proj, ld_proj, ld_rot, r0, nr, rotinv,
                                   use_floor, floor_v, has_scale, scale, weight, p, xr, ratio, part,
                                   fpart, direct, st, stage, fout, ld_fout, gin, ld_gin);
        break;
    }
    if (rc != JSCC_OK) return rc;
  }
  return JSCC_OK;
}

template <typename T>
static int sc_sensitivity_typed(const T* A, int64_t lda, const int64_t* row_idx, int64_t n_bins, int64_t V,
                                int n_rot, const int64_t* rotinv, int64_t ld_rot, float* weight, int64_t col_tiles,
                                int64_t chunks, int64_t rows_per_chunk, int64_t ldp, float* sum, float* comp,
                                cudaStream_t st) {
  constexpr int NV = VecTraits<T>::kVec;
  const bool vec_ok = ((lda * (int64_t)sizeof(T)) % 16 == 0) && (reinterpret_cast<uintptr_t>(A) % 16 == 0);
  const int sms = num_sms();
  dim3 grid((unsigned)col_tiles, (unsigned)chunks);
  const int threads = kColTile / NV;
  JSCC_TIMED("sc_colsum_kahan", st, {
    if (vec_ok)
      sc_colsum_kahan_kernel<T, true><<<grid, threads, 0, st>>>(A, lda, row_idx, n_bins, V, rows_per_chunk, sum,
                                                                comp, ldp);
    else
      sc_colsum_kahan_kernel<T, false><<<grid, threads, 0, st>>>(A, lda, row_idx, n_bins, V, rows_per_chunk, sum,
                                                                 comp, ldp);
  });
  JSCC_LAUNCH_CHECK();
  int64_t blocks = (V + 255) / 256;
  if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
  if (blocks < 1) blocks = 1;
  JSCC_TIMED("sc_sensitivity", st,
             sc_sensitivity_kernel<<<(unsigned)blocks, 256, 0, st>>>(sum, comp, ldp, (int)chunks, rotinv, ld_rot,
                                                                     n_rot, V, weight));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

// ------------------------------------------------------------------ FP64 evaluation
// Reference-grade projector halves for gradient checks (sums in double; not a hot path).
// f[b, r] = sum_j A[rb, j] x[rot[j, r] - 1]: one warp per (b, r).
template <typename T>
__global__ void sc_project_f64_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx,
                                      int64_t n_bins, int64_t V, int n_rot, const double* __restrict__ x,
                                      const int64_t* __restrict__ rotmat, int64_t ld_rot, double* __restrict__ out,
                                      int64_t ld_out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < n_bins * n_rot; w += warps) {
    const int64_t b = w / n_rot;
    const int r = (int)(w % n_rot);
    const T* row = A + (row_idx ? row_idx[b] : b) * lda;
    double acc = 0.0;
    for (int64_t j = lane; j < V; j += 32) {
      int64_t src = j;
      if (rotmat) {
        src = rotmat[j * ld_rot + r] - 1;
        if (src < 0 || src >= V) {
          atomicAdd(&g_bad_index_count, 1u);
          continue;
        }
      }
      acc += (double)load_elem(row, j) * x[src];
    }
    acc = warp_sum_d(acc);
    if (lane == 0) out[b * ld_out + r] = acc;
  }
}

// u[r][c] = sum_b A[rb, c] g[b, r]
template <typename T>
__global__ void sc_colsum_f64_kernel(const T* __restrict__ A, int64_t lda, const int64_t* __restrict__ row_idx,
                                     int64_t n_bins, int64_t V, int n_rot, const double* __restrict__ g, int64_t ld_g,
                                     double* __restrict__ u) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < V * n_rot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / V);
    const int64_t c = t % V;
    double acc = 0.0;
    for (int64_t b = 0; b < n_bins; ++b) acc += (double)load_elem(A + (row_idx ? row_idx[b] : b) * lda, c) * g[b * ld_g + r];
    u[(int64_t)r * V + c] = acc;
  }
}

// weight[j] += scale * sum_r u[r][rotinv[j, r] - 1]
__global__ void sc_gather_f64_kernel(const double* __restrict__ u, int64_t V, int n_rot,
                                     const int64_t* __restrict__ rotinv, int64_t ld_rot, double scale,
                                     double* __restrict__ weight) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V; j += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int r = 0; r < n_rot; ++r) {
      int64_t src = j;
      if (rotinv) {
        src = rotinv[j * ld_rot + r] - 1;
        if (src < 0 || src >= V) {
          atomicAdd(&g_bad_index_count, 1u);
          continue;
        }
      }
      acc += u[(int64_t)r * V + src];
    }
    weight[j] += scale * acc;
  }
}

}  // namespace jscc

using namespace jscc;

extern "C" {

int jscc_sc_sensitivity(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx, int64_t n_bins,
                        int64_t n_vox, int32_t n_rot, const int64_t* rotmat_inv, int64_t ld_rot, float* weight,
                        void* workspace, size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0, "jscc_sc_sensitivity: negative size");
  JSCC_REQUIRE(n_rot >= 1, "jscc_sc_sensitivity: n_rot must be >= 1 (got %d)", n_rot);
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16, "jscc_sc_sensitivity: unsupported a_dtype %d",
               a_dtype);
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(A && weight, "jscc_sc_sensitivity: null pointer argument");
  JSCC_REQUIRE(lda >= n_vox, "jscc_sc_sensitivity: lda (%lld) < n_vox (%lld)", (long long)lda, (long long)n_vox);
  JSCC_REQUIRE(rotmat_inv != nullptr || n_rot == 1, "jscc_sc_sensitivity: n_rot > 1 needs rotmat_inv");
  JSCC_REQUIRE(rotmat_inv == nullptr || ld_rot >= n_rot, "jscc_sc_sensitivity: ld_rot (%lld) < n_rot (%d)",
               (long long)ld_rot, n_rot);
  const ScPlan p = plan_sc(n_bins, n_vox, 1);
  JSCC_REQUIRE(workspace != nullptr && workspace_bytes >= p.ws_bytes,
               "jscc_sc_sensitivity: workspace too small (%zu < %zu bytes)", workspace_bytes, p.ws_bytes);
  // compensated sums: half as many row chunks as the back pass, so the sums and their carried
  // errors (2 x chunks x ldx floats) fit in the same workspace (>= (chunks + 1) x ldx floats)
  int64_t chunks = (p.chunks + 1) / 2;
  if (chunks < 1) chunks = 1;
  const int64_t rows_per_chunk = (n_bins + chunks - 1) / chunks;
  chunks = (n_bins + rows_per_chunk - 1) / rows_per_chunk;
  Carver cv(workspace, workspace_bytes);
  float* sum = cv.take<float>((size_t)chunks * p.ldx);
  float* comp = cv.take<float>((size_t)chunks * p.ldx);
  JSCC_REQUIRE(cv.ok(), "jscc_sc_sensitivity: workspace carve overflow");
  cudaStream_t st = as_stream(stream);
  if (a_dtype == JSCC_DTYPE_F32)
    return sc_sensitivity_typed<float>(static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, n_rot, rotmat_inv,
                                       ld_rot, weight, p.col_tiles, chunks, rows_per_chunk, p.ldx, sum, comp, st);
  return sc_sensitivity_typed<__nv_bfloat16>(static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins, n_vox,
                                             n_rot, rotmat_inv, ld_rot, weight, p.col_tiles, chunks, rows_per_chunk,
                                             p.ldx, sum, comp, st);
}

size_t jscc_sc_weight_workspace_bytes(int64_t n_bins, int64_t n_vox, int32_t n_rot) {
  const ScPlan p = plan_sc(n_bins, n_vox, n_rot);
  return p.ws_bytes + p.fs_bytes;
}

int jscc_sc_weight(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox,
                   const float* proj, int64_t ld_proj, int32_t n_rot, const float* img,
                   const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot,
                   int32_t use_floor, float floor_v, float scale, float* weight, void* workspace,
                   size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0, "jscc_sc_weight: negative size");
  JSCC_REQUIRE(n_rot >= 1, "jscc_sc_weight: n_rot must be >= 1 (got %d)", n_rot);
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16,
               "jscc_sc_weight: unsupported a_dtype %d", a_dtype);
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;  // nothing to add
  JSCC_REQUIRE(A && proj && img && weight, "jscc_sc_weight: null pointer argument");
  JSCC_REQUIRE(lda >= n_vox, "jscc_sc_weight: lda (%lld) < n_vox (%lld)", (long long)lda,
               (long long)n_vox);
  JSCC_REQUIRE(ld_proj >= n_rot, "jscc_sc_weight: ld_proj (%lld) < n_rot (%d)",
               (long long)ld_proj, n_rot);
  JSCC_REQUIRE((rotmat == nullptr && rotmat_inv == nullptr) || ld_rot >= n_rot,
               "jscc_sc_weight: ld_rot (%lld) < n_rot (%d)", (long long)ld_rot, n_rot);
  const ScPlan p = plan_sc(n_bins, n_vox, n_rot);
  JSCC_REQUIRE(workspace != nullptr && workspace_bytes >= p.ws_bytes,
               "jscc_sc_weight: workspace too small (%zu < %zu bytes)", workspace_bytes,
               p.ws_bytes);
  Carver cv(workspace, workspace_bytes);
  float* xr = cv.take<float>((size_t)p.rb * p.ldx);
  float* ratio = cv.take<float>((size_t)n_bins * p.rb);
  float* part = cv.take<float>((size_t)p.chunks * p.rb * p.ldx);
  float* fpart = cv.take<float>((size_t)p.fwd_warps * p.fwd_maxp * p.rb);
  JSCC_REQUIRE(cv.ok(), "jscc_sc_weight: workspace carve overflow");
  float* fs_part = fused_partials(p, cv);
  const int has_scale = scale != 1.0f;
  cudaStream_t st = as_stream(stream);
  if (a_dtype == JSCC_DTYPE_F32)
    return sc_weight_typed<float>(static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, proj,
                                  ld_proj,
                                  n_rot, img, rotmat, rotmat_inv, ld_rot, use_floor, floor_v, has_scale,
                                  scale, weight, p, xr, ratio, part, fpart, st, 0, nullptr, 0, nullptr, 0,
                                  fs_part);
  return sc_weight_typed<__nv_bfloat16>(static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins,
                                        n_vox,
                                        proj, ld_proj, n_rot, img, rotmat, rotmat_inv, ld_rot, use_floor,
                                        floor_v, has_scale, scale, weight, p, xr, ratio, part, fpart, st, 0, nullptr,
                                        0, nullptr, 0, fs_part);
}

// The two halves of jscc_sc_weight on their own (the differentiable projector's forward and
// backward): out[b * ld_out + r] = A[rb] . rot_r(img), and weight += scale * sum_r
// rotinv_r(A^T g[:, r]). Same workspace as jscc_sc_weight for the same sizes.
static int sc_stage_entry(const char* what, int stage, const void* A, int32_t a_dtype, int64_t lda,
                          const int64_t* row_idx, int64_t n_bins, int64_t n_vox, int32_t n_rot, const float* img,
                          const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, float* out,
                          int64_t ld_out, const float* g, int64_t ld_g, float scale, float* weight, void* workspace,
                          size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0, "%s: negative size", what);
  JSCC_REQUIRE(n_rot >= 1, "%s: n_rot must be >= 1 (got %d)", what, n_rot);
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16, "%s: unsupported a_dtype %d", what, a_dtype);
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(A, "%s: null matrix", what);
  JSCC_REQUIRE(lda >= n_vox, "%s: lda (%lld) < n_vox (%lld)", what, (long long)lda, (long long)n_vox);
  if (stage == 1) {
    JSCC_REQUIRE(img && out && ld_out >= n_rot, "%s: null image/output or ld_out < n_rot", what);
    JSCC_REQUIRE(rotmat != nullptr || n_rot == 1, "%s: n_rot > 1 needs rotmat", what);
  } else {
    JSCC_REQUIRE(g && weight && ld_g >= n_rot, "%s: null input/weight or ld_g < n_rot", what);
    JSCC_REQUIRE(rotmat_inv != nullptr || n_rot == 1, "%s: n_rot > 1 needs rotmat_inv", what);
  }
  JSCC_REQUIRE(ld_rot >= n_rot || (rotmat == nullptr && rotmat_inv == nullptr), "%s: ld_rot < n_rot", what);
  const ScPlan p = plan_sc(n_bins, n_vox, n_rot);
  JSCC_REQUIRE(workspace != nullptr && workspace_bytes >= p.ws_bytes, "%s: workspace too small (%zu < %zu bytes)",
               what, workspace_bytes, p.ws_bytes);
  Carver cv(workspace, workspace_bytes);
  float* xr = cv.take<float>((size_t)p.rb * p.ldx);
  float* ratio = cv.take<float>((size_t)n_bins * p.rb);
  float* part = cv.take<float>((size_t)p.chunks * p.rb * p.ldx);
  float* fpart = cv.take<float>((size_t)p.fwd_warps * p.fwd_maxp * p.rb);
  JSCC_REQUIRE(cv.ok(), "%s: workspace carve overflow", what);
  const int has_scale = scale != 1.0f;
  cudaStream_t st = as_stream(stream);
  if (a_dtype == JSCC_DTYPE_F32)
    return sc_weight_typed<float>(static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, nullptr, 0, n_rot, img,
                                  rotmat, rotmat_inv, ld_rot, 0, 0.f, has_scale, scale, weight, p, xr, ratio, part,
                                  fpart, st, stage, out, ld_out, g, ld_g);
  return sc_weight_typed<__nv_bfloat16>(static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins, n_vox, nullptr,
                                        0, n_rot, img, rotmat, rotmat_inv, ld_rot, 0, 0.f, has_scale, scale, weight, p,
                                        xr, ratio, part, fpart, st, stage, out, ld_out, g, ld_g);
}

int jscc_sc_project(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx, int64_t n_bins,
                    int64_t n_vox, int32_t n_rot, const float* img, const int64_t* rotmat, int64_t ld_rot, float* out,
                    int64_t ld_out, void* workspace, size_t workspace_bytes, void* stream) {
  return sc_stage_entry("jscc_sc_project", 1, A, a_dtype, lda, row_idx, n_bins, n_vox, n_rot, img, rotmat, nullptr,
                        ld_rot, out, ld_out, nullptr, 0, 1.f, nullptr, workspace, workspace_bytes, stream);
}

int jscc_sc_backproject(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx, int64_t n_bins,
                        int64_t n_vox, int32_t n_rot, const float* g, int64_t ld_g, const int64_t* rotmat_inv,
                        int64_t ld_rot, float scale, float* weight, void* workspace, size_t workspace_bytes,
                        void* stream) {
  return sc_stage_entry("jscc_sc_backproject", 2, A, a_dtype, lda, row_idx, n_bins, n_vox, n_rot, nullptr, nullptr,
                        rotmat_inv, ld_rot, nullptr, 0, g, ld_g, scale, weight, workspace, workspace_bytes, stream);
}

size_t jscc_sc_f64_workspace_bytes(int64_t n_vox, int32_t n_rot) {
  return align_up((size_t)(n_vox > 0 ? n_vox : 1) * (size_t)(n_rot > 0 ? n_rot : 1) * sizeof(double), 256) + 256;
}

int jscc_sc_project_f64(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx, int64_t n_bins,
                        int64_t n_vox, int32_t n_rot, const double* img, const int64_t* rotmat, int64_t ld_rot,
                        double* out, int64_t ld_out, void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0 && n_rot >= 1, "jscc_sc_project_f64: bad sizes");
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16, "jscc_sc_project_f64: bad a_dtype");
  JSCC_REQUIRE(rotmat != nullptr || n_rot == 1, "jscc_sc_project_f64: n_rot > 1 needs rotmat");
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(A && img && out && lda >= n_vox && ld_out >= n_rot, "jscc_sc_project_f64: bad argument");
  cudaStream_t st = as_stream(stream);
  int64_t blocks = (n_bins * n_rot + 7) / 8;  // 8 warps per block
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  if (a_dtype == JSCC_DTYPE_F32)
    JSCC_TIMED("sc_project_f64", st,
               (sc_project_f64_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
                   static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, n_rot, img, rotmat, ld_rot, out, ld_out)));
  else
    JSCC_TIMED("sc_project_f64", st,
               (sc_project_f64_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, st>>>(
                   static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins, n_vox, n_rot, img, rotmat, ld_rot, out,
                   ld_out)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_sc_backproject_f64(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx, int64_t n_bins,
                            int64_t n_vox, int32_t n_rot, const double* g, int64_t ld_g, const int64_t* rotmat_inv,
                            int64_t ld_rot, double scale, double* weight, void* workspace, size_t workspace_bytes,
                            void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0 && n_rot >= 1, "jscc_sc_backproject_f64: bad sizes");
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16, "jscc_sc_backproject_f64: bad a_dtype");
  JSCC_REQUIRE(rotmat_inv != nullptr || n_rot == 1, "jscc_sc_backproject_f64: n_rot > 1 needs rotmat_inv");
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(A && g && weight && lda >= n_vox && ld_g >= n_rot, "jscc_sc_backproject_f64: bad argument");
  JSCC_REQUIRE(workspace && workspace_bytes >= jscc_sc_f64_workspace_bytes(n_vox, n_rot),
               "jscc_sc_backproject_f64: workspace too small");
  Carver cv(workspace, workspace_bytes);
  double* u = cv.take<double>((size_t)n_vox * n_rot);
  JSCC_REQUIRE(cv.ok(), "jscc_sc_backproject_f64: workspace carve overflow");
  cudaStream_t st = as_stream(stream);
  int64_t blocks = (n_vox * n_rot + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  if (a_dtype == JSCC_DTYPE_F32)
    JSCC_TIMED("sc_colsum_f64", st,
               (sc_colsum_f64_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
                   static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, n_rot, g, ld_g, u)));
  else
    JSCC_TIMED("sc_colsum_f64", st,
               (sc_colsum_f64_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, st>>>(
                   static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins, n_vox, n_rot, g, ld_g, u)));
  JSCC_LAUNCH_CHECK();
  blocks = (n_vox + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  JSCC_TIMED("sc_gather_f64", st,
             (sc_gather_f64_kernel<<<(unsigned)blocks, 256, 0, st>>>(u, n_vox, n_rot, rotmat_inv, ld_rot, scale,
                                                                     weight)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_take_bad_index_count(unsigned int* out) {
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_bad_index_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_bad_index_count, &zero, sizeof(zero)));
  h += jscc::take_prior_bad_index_count();
  if (out) *out = h;
  return JSCC_OK;
}

}  // extern "C"

// ============================================================================
// No-allocation variant of jscc_sc_weight.
//
// Some callers cannot hand this library a workspace: a host framework that owns all
// device memory through its own pool and forbids allocations from plugins, a language
// runtime driving the library through a bare FFI without any device allocator, or a
// latency-critical loop that must not pay cudaMalloc's implicit synchronisation. For
// them the scratch of the SC weight lives in one fixed file-scope device array,
// allocated when the library's device code is loaded on a GPU and held until the
// process exits.
//
// The array's name is only a host-side stand-in in host code: its device address is
// obtained once per device with cudaGetSymbolAddress (the first call on each device
// does this, with that device current) and that address is what the kernels get.
// Every call shares the one array: calls that may overlap on the GPU (different
// streams, or concurrent host threads) race on it and must be serialised by the
// caller. No byte of the scratch needs to start at zero: each call writes every
// scratch element before it reads it.
// ============================================================================

namespace jscc {

static __device__ __align__(256) unsigned char g_sc_noalloc_scratch[JSCC_SC_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch_address(void** out) {
  int dev = -1;
  JSCC_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("jscc_sc_weight_noalloc: device ordinal %d outside the supported range", dev);
    return JSCC_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sc_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("jscc_sc_weight_noalloc: cudaGetSymbolAddress of the scratch array failed on device %d: %s",
                dev, cudaGetErrorString(e));
      return JSCC_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return JSCC_OK;
}

}  // namespace jscc

extern "C" int jscc_sc_weight_noalloc(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                                      int64_t n_bins, int64_t n_vox, const float* proj, int64_t ld_proj,
                                      int32_t n_rot, const float* img, const int64_t* rotmat,
                                      const int64_t* rotmat_inv, int64_t ld_rot, int32_t use_floor,
                                      float floor_v, float scale, float* weight, void* stream) {
  JSCC_REQUIRE(n_bins >= 0 && n_vox >= 0, "jscc_sc_weight_noalloc: negative size");
  JSCC_REQUIRE(n_rot >= 1, "jscc_sc_weight_noalloc: n_rot must be >= 1 (got %d)", n_rot);
  JSCC_REQUIRE(a_dtype == JSCC_DTYPE_F32 || a_dtype == JSCC_DTYPE_BF16,
               "jscc_sc_weight_noalloc: unsupported a_dtype %d", a_dtype);
  if (n_bins == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(A && proj && img && weight, "jscc_sc_weight_noalloc: null pointer argument");
  JSCC_REQUIRE(lda >= n_vox, "jscc_sc_weight_noalloc: lda (%lld) < n_vox (%lld)", (long long)lda,
               (long long)n_vox);
  JSCC_REQUIRE(ld_proj >= n_rot, "jscc_sc_weight_noalloc: ld_proj (%lld) < n_rot (%d)",
               (long long)ld_proj, n_rot);
  JSCC_REQUIRE((rotmat == nullptr && rotmat_inv == nullptr) || ld_rot >= n_rot,
               "jscc_sc_weight_noalloc: ld_rot (%lld) < n_rot (%d)", (long long)ld_rot, n_rot);
  const ScPlan p = plan_sc(n_bins, n_vox, n_rot);
  JSCC_REQUIRE(p.ws_bytes <= (size_t)JSCC_SC_NOALLOC_SCRATCH_BYTES,
               "jscc_sc_weight_noalloc: this problem (%lld bins x %lld voxels, %d rotations) needs %zu "
               "bytes of scratch but the fixed scratch array holds %zu bytes; call jscc_sc_weight with a "
               "caller-provided workspace instead",
               (long long)n_bins, (long long)n_vox, n_rot, p.ws_bytes,
               (size_t)JSCC_SC_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  const int rc = noalloc_scratch_address(&scratch);
  if (rc != JSCC_OK) return rc;
  Carver cv(scratch, (size_t)JSCC_SC_NOALLOC_SCRATCH_BYTES);
  float* xr = cv.take<float>((size_t)p.rb * p.ldx);
  float* ratio = cv.take<float>((size_t)n_bins * p.rb);
  float* part = cv.take<float>((size_t)p.chunks * p.rb * p.ldx);
  float* fpart = cv.take<float>((size_t)p.fwd_warps * p.fwd_maxp * p.rb);
  JSCC_REQUIRE(cv.ok(), "jscc_sc_weight_noalloc: scratch carve overflow");
  float* fs_part = fused_partials(p, cv);
  const int has_scale = scale != 1.0f;
  cudaStream_t st = as_stream(stream);
  if (a_dtype == JSCC_DTYPE_F32)
    return sc_weight_typed<float>(static_cast<const float*>(A), lda, row_idx, n_bins, n_vox, proj, ld_proj,
                                  n_rot, img, rotmat, rotmat_inv, ld_rot, use_floor, floor_v, has_scale, scale,
                                  weight, p, xr, ratio, part, fpart, st, 0, nullptr, 0, nullptr, 0, fs_part);
  return sc_weight_typed<__nv_bfloat16>(static_cast<const __nv_bfloat16*>(A), lda, row_idx, n_bins, n_vox,
                                        proj, ld_proj, n_rot, img, rotmat, rotmat_inv, ld_rot, use_floor,
                                        floor_v, has_scale, scale, weight, p, xr, ratio, part, fpart, st, 0, nullptr,
                                        0, nullptr, 0, fs_part);
}
