// Sparse Compton rows on a coarse polar grid (kernel c): separable coarse<->fine maps,
// pack/unpack, materialisation and the fused sparse list-mode weight.
//
// Reference semantics: compton_sparse_ops.py. The reference applies its operators as
// dense matrix products (layer_expand is [fine layers x coarse layers] block-diagonal,
// z_expand [fine z x coarse z]); every row of those matrices has at most two non-zeros
// (two-tap periodic interpolation in theta, two-tap linear interpolation in z), and the
// reduce matrices sample (theta) or interpolate (z). Here each map is a pair of small CSR
// tables built from the reference's own matrices by the host, so each output element
// costs a handful of loads instead of a full matrix row: O(V) per row instead of O(V_f V_c).
//
// out[r][zo * n_lo + lo] = sum_{(zi, wz) in Z[zo]} wz * sum_{(li, wl) in L[lo]} wl * in[r][zi * n_li + li]
// (layer sum first, then z, as the reference's two matmuls).
#include <climits>
#include "jscc_common.cuh"

#include <algorithm>
#include <type_traits>

namespace jscc {

// ------------------------------------------------------------------ separable map
template <typename TI>
__device__ __forceinline__ float ld_any(const TI* p, int64_t i);
template <>
__device__ __forceinline__ float ld_any<float>(const float* p, int64_t i) { return __ldg(p + i); }
// plain conversions (usable on shared-memory values)
__device__ __forceinline__ float to_float(float v) { return v; }
__device__ __forceinline__ float to_float(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ float ld_any<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

template <typename TI>
__global__ void sparse_map_kernel(const TI* __restrict__ in, int64_t ld_in, const int32_t* __restrict__ row_idx,
                                  int64_t n_rows, float* __restrict__ out, int64_t ld_out,
                                  const int32_t* __restrict__ zp, const int32_t* __restrict__ zi,
                                  const float* __restrict__ zw, int n_zo, const int32_t* __restrict__ lp,
                                  const int32_t* __restrict__ li, const float* __restrict__ lw, int n_lo, int n_li) {
  const int64_t r = blockIdx.y;
  if (r >= n_rows) return;
  const TI* src = in + (row_idx ? (int64_t)row_idx[r] : r) * ld_in;
  const int64_t n_out = (int64_t)n_zo * n_lo;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out; o += (int64_t)gridDim.x * blockDim.x) {
    const int zo = (int)(o / n_lo), lo = (int)(o % n_lo);
    float acc = 0.f;
    for (int a = zp[zo]; a < zp[zo + 1]; ++a) {
      const int64_t base = (int64_t)zi[a] * n_li;
      float s = 0.f;
      for (int b = lp[lo]; b < lp[lo + 1]; ++b) s = fmaf(lw[b], ld_any(src, base + li[b]), s);
      acc = fmaf(zw[a], s, acc);
    }
    out[r * ld_out + o] = acc;
  }
}

// ------------------------------------------------------------------ pack / unpack
__global__ void sparse_pack_kernel(const int64_t* __restrict__ cp1, const float* __restrict__ tc, int64_t ld_tc,
                                   int64_t n, int64_t vc, float* __restrict__ out, int64_t ld_out) {
  const int64_t i = blockIdx.y;
  if (i >= n) return;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c <= vc; c += (int64_t)gridDim.x * blockDim.x)
    out[i * ld_out + c] = c == 0 ? (float)cp1[i] : tc[i * ld_tc + c - 1];
}

__global__ void sparse_unpack_kernel(const float* __restrict__ rows, int64_t ld_rows, int64_t n,
                                     int64_t* __restrict__ cp1) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    cp1[i] = (int64_t)rintf(rows[i * ld_rows]);  // torch.round: half to even
}

// ------------------------------------------------------------------ fine value of a sparse row
// Upsample taps: fine j = zf * n_lf + lf has z taps (zt[2 zf], zt[2 zf + 1]) with weights
// zwt[...] and layer taps (lt[2 lf], lt[2 lf + 1]) with weights lwt[...]; a missing tap has
// weight 0 and a valid index.
struct UpTaps {
  const int32_t* zt;
  const float* zwt;
  const int32_t* lt;
  const float* lwt;
  int n_lf;
  int n_lc;
};

template <typename TC>
__device__ __forceinline__ float up_value(const TC* __restrict__ tc, const UpTaps& t, int zf, int lf) {
  const int l0 = t.lt[2 * lf], l1 = t.lt[2 * lf + 1];
  const float w0 = t.lwt[2 * lf], w1 = t.lwt[2 * lf + 1];
  const int z0 = t.zt[2 * zf], z1 = t.zt[2 * zf + 1];
  const float u0 = t.zwt[2 * zf], u1 = t.zwt[2 * zf + 1];
  const TC* r0 = tc + (int64_t)z0 * t.n_lc;
  const TC* r1 = tc + (int64_t)z1 * t.n_lc;
  float a = w0 * ld_any(r0, l0);
  if (w1 != 0.f) a = fmaf(w1, ld_any(r0, l1), a);
  float v = u0 * a;
  if (u1 != 0.f) {
    float b = w0 * ld_any(r1, l0);
    if (w1 != 0.f) b = fmaf(w1, ld_any(r1, l1), b);
    v = fmaf(u1, b, v);
  }
  return v;
}

// The same two-tap upsample from a coarse row held in SHARED memory (plain loads: the
// read-only global path of ld_any must not be used on a shared-memory address).
__device__ __forceinline__ float up_value_shared(const float* tc, const UpTaps& t, int zf, int lf) {
  const int l0 = t.lt[2 * lf], l1 = t.lt[2 * lf + 1];
  const float w0 = t.lwt[2 * lf], w1 = t.lwt[2 * lf + 1];
  const int z0 = t.zt[2 * zf], z1 = t.zt[2 * zf + 1];
  const float u0 = t.zwt[2 * zf], u1 = t.zwt[2 * zf + 1];
  const float* r0 = tc + (int64_t)z0 * t.n_lc;
  const float* r1 = tc + (int64_t)z1 * t.n_lc;
  float a = w0 * r0[l0];
  if (w1 != 0.f) a = fmaf(w1, r0[l1], a);
  float v = u0 * a;
  if (u1 != 0.f) {
    float b = w0 * r1[l0];
    if (w1 != 0.f) b = fmaf(w1, r1[l1], b);
    v = fmaf(u1, b, v);
  }
  return v;
}

// Event rows in either layout: packed float rows (cp1 as float in column 0, the
// reference's format) or split storage (0-based sysmat row ids + coarse rows of TC,
// float32 or bf16 — bf16 cannot hold the ids, hence the split).
template <typename TC>
struct SpRows {
  const float* packed;   // non-null: packed layout
  const int32_t* ids;    // split layout: row ids (0-based, clamped on use)
  const TC* tc;          // split layout: coarse rows
  int64_t ld;            // row stride (elements)
  int64_t n_det;
  __device__ __forceinline__ int64_t row_of(int64_t i) const {
    int64_t g = packed ? (int64_t)rintf(packed[i * ld]) - 1 : (int64_t)ids[i];
    return g < 0 ? 0 : (g >= n_det ? n_det - 1 : g);
  }
  __device__ __forceinline__ const TC* coarse(int64_t i) const;
};
template <>
__device__ __forceinline__ const float* SpRows<float>::coarse(int64_t i) const {
  return packed ? packed + i * ld + 1 : tc + i * ld;
}
template <>
__device__ __forceinline__ const __nv_bfloat16* SpRows<__nv_bfloat16>::coarse(int64_t i) const {
  return tc + i * ld;
}

__device__ __forceinline__ float finite_or_zero(float v) { return isfinite(v) ? v : 0.f; }

// a sysmat row index clamped into [0, n_det)
__device__ __forceinline__ int64_t clamp_row(int64_t g, int64_t n_det) {
  return g < 0 ? 0 : (g >= n_det ? n_det - 1 : g);
}

// ------------------------------------------------------------------ materialise
// fine[i][j] = nan_to_num(up(tc_i)[j] * sysmat[clamp(cp1_i - 1)][j]); rsum[i] = sum_j fine[i][j]
template <typename TE>
__global__ void __launch_bounds__(256)
sparse_materialize_kernel(const float* __restrict__ rows, int64_t ld_rows, int64_t n, int64_t vf,
                          const TE* __restrict__ eff, int64_t ld_eff, int64_t n_det, UpTaps taps,
                          float* __restrict__ fine, int64_t ld_fine, float* __restrict__ rsum) {
  __shared__ float red[8];
  const int64_t i = blockIdx.x;
  if (i >= n) return;
  const float* row = rows + i * ld_rows;
  int64_t g = (int64_t)rintf(row[0]) - 1;
  g = g < 0 ? 0 : (g >= n_det ? n_det - 1 : g);
  const float* tc = row + 1;
  const TE* er = eff + g * ld_eff;
  float s = 0.f;
  for (int64_t j = threadIdx.x; j < vf; j += blockDim.x) {
    const int zf = (int)(j / taps.n_lf), lf = (int)(j % taps.n_lf);
    const float v = finite_or_zero(up_value<float>(tc, taps, zf, lf) * ld_any(er, j));
    fine[i * ld_fine + j] = v;
    s += v;
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    rsum[i] = t;
  }
}

// ------------------------------------------------------------------ fused sparse weight
constexpr int kSpThreads = 256;

// f[i] = sum_j v_ij x_j, s[i] = sum_j v_ij, v = up(tc_i) * eff_g(i) (nan_to_num in MATERIALIZE mode)
template <int EB, bool MATERIALIZE, typename TE, typename TC>
__global__ void __launch_bounds__(kSpThreads)
sparse_forward_kernel(SpRows<TC> rows, int64_t n, int64_t vf, const float* __restrict__ x,
                      const TE* __restrict__ eff, int64_t ld_eff, UpTaps taps, float* __restrict__ f_out,
                      float* __restrict__ s_out) {
  __shared__ int64_t sg[EB];
  __shared__ float red[kSpThreads / 32][2 * EB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t i0 = (int64_t)blockIdx.x * EB;
  const int ne = (n - i0) < EB ? (int)(n - i0) : EB;
  if (tid < EB) {
    const int64_t i = i0 + tid < n ? i0 + tid : n - 1;
    sg[tid] = rows.row_of(i);
  }
  __syncthreads();
  float af[EB], as[EB];
#pragma unroll
  for (int e = 0; e < EB; ++e) af[e] = as[e] = 0.f;
  for (int64_t j = tid; j < vf; j += kSpThreads) {
    const int zf = (int)(j / taps.n_lf), lf = (int)(j % taps.n_lf);
    const float xj = __ldg(x + j);
#pragma unroll
    for (int e = 0; e < EB; ++e) {
      if (e < ne) {
        float v = up_value<TC>(rows.coarse(i0 + e), taps, zf, lf);
        if (v != 0.f) {
          v *= ld_any(eff + sg[e] * ld_eff, j);
          if (MATERIALIZE) v = finite_or_zero(v);
          af[e] = fmaf(v, xj, af[e]);
          as[e] += v;
        }
      }
    }
  }
#pragma unroll
  for (int e = 0; e < EB; ++e) {
    const float a = warp_sum(af[e]);
    const float b = warp_sum(as[e]);
    if (lane == 0) {
      red[warp][e] = a;
      red[warp][EB + e] = b;
    }
  }
  __syncthreads();
  if (tid < ne) {
    float fa = 0.f, sa = 0.f;
#pragma unroll
    for (int w = 0; w < kSpThreads / 32; ++w) {
      fa += red[w][tid];
      sa += red[w][EB + tid];
    }
    f_out[i0 + tid] = fa;
    s_out[i0 + tid] = sa;
  }
}

// coef[i]: MATERIALIZE: valid = isfinite(s) && s > 0; coef = (1 / max(f / s, 1e-12)) / s, else 0
//          GROUPED:     coef = 1 / max(f, 1e-12)
template <bool MATERIALIZE>
__global__ void sparse_coef_kernel(const float* __restrict__ f, const float* __restrict__ s, int64_t n,
                                   float* __restrict__ coef) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (MATERIALIZE) {
      const float si = s[i];
      const bool valid = isfinite(si) && si > 0.f;
      coef[i] = valid ? (1.0f / fmaxf(f[i] / si, 1e-12f)) / si : 0.f;
    } else {
      coef[i] = 1.0f / fmaxf(f[i], 1e-12f);
    }
  }
}

constexpr int kSpStage = 64;

// part[chunk][j] = sum_{i in chunk} v_ij coef_i
template <bool MATERIALIZE, typename TE, typename TC>
__global__ void __launch_bounds__(kSpThreads)
sparse_back_kernel(SpRows<TC> rows, int64_t n, int64_t ev_per_chunk, int64_t vf, const float* __restrict__ coef,
                   const TE* __restrict__ eff, int64_t ld_eff, UpTaps taps, float* __restrict__ part, int64_t ldp) {
  __shared__ int64_t sg[kSpStage];
  __shared__ float sc[kSpStage];
  const int tid = threadIdx.x;
  const int64_t j = (int64_t)blockIdx.x * kSpThreads + tid;
  const int64_t e_begin = (int64_t)blockIdx.y * ev_per_chunk;
  int64_t e_end = e_begin + ev_per_chunk;
  if (e_end > n) e_end = n;
  const int zf = j < vf ? (int)(j / taps.n_lf) : 0, lf = j < vf ? (int)(j % taps.n_lf) : 0;
  float acc = 0.f;
  for (int64_t s0 = e_begin; s0 < e_end; s0 += kSpStage) {
    const int cnt = (e_end - s0) < kSpStage ? (int)(e_end - s0) : kSpStage;
    __syncthreads();
    if (tid < cnt) {
      sg[tid] = rows.row_of(s0 + tid);
      sc[tid] = coef[s0 + tid];
    }
    __syncthreads();
    if (j < vf) {
      for (int e = 0; e < cnt; ++e) {
        const float ce = sc[e];
        if (ce == 0.f) continue;
        float v = up_value<TC>(rows.coarse(s0 + e), taps, zf, lf);
        if (v != 0.f) {
          v *= ld_any(eff + sg[e] * ld_eff, j);
          if (MATERIALIZE) v = finite_or_zero(v);
          acc = fmaf(v, ce, acc);
        }
      }
    }
  }
  if (j < vf) part[(int64_t)blockIdx.y * ldp + j] = acc;
}

// weight[j] += scale * nan_to_num(sum_c part[c][src(j)]), src = rotmat_inv[j, 0] - 1 or j
__global__ void sparse_reduce_kernel(const float* __restrict__ part, int64_t ldp, int chunks,
                                     const int64_t* __restrict__ rotinv, int64_t ld_rot, int64_t V, int has_scale,
                                     float scale, float* __restrict__ weight) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t src = j;
    if (rotinv) {
      src = rotinv[j * ld_rot] - 1;
      if (src < 0 || src >= V) continue;
    }
    float s = 0.f;
    for (int c = 0; c < chunks; ++c) s += part[(int64_t)c * ldp + src];
    s = finite_or_zero(s);
    weight[j] = has_scale ? __fadd_rn(weight[j], __fmul_rn(scale, s)) : __fadd_rn(weight[j], s);
  }
}

// Shared with sc_projector.cu.
__global__ void sc_gather_rot_kernel(const float* __restrict__ img, const int64_t* __restrict__ rotmat,
                                     int64_t ld_rot, int r0, int nr, int64_t V, int64_t ldx,
                                     float* __restrict__ xr);

struct SpPlan {
  int64_t chunks, ev_per_chunk, ldp;
  size_t ws_bytes;
};

static SpPlan plan_sparse(int64_t n, int64_t vf) {
  SpPlan p{};
  const int64_t tiles = (vf + kSpThreads - 1) / kSpThreads;
  int64_t chunks = (2432 + tiles - 1) / (tiles > 0 ? tiles : 1);
  const int64_t max_chunks = (n + 63) / 64;
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks < 1) chunks = 1;
  p.ev_per_chunk = (n + chunks - 1) / chunks;
  if (p.ev_per_chunk < 1) p.ev_per_chunk = 1;
  p.chunks = (n + p.ev_per_chunk - 1) / p.ev_per_chunk;
  if (p.chunks < 1) p.chunks = 1;
  p.ldp = (int64_t)align_up((size_t)(vf > 0 ? vf : 1), 8);
  size_t b = 0;
  b += align_up((size_t)p.ldp * sizeof(float), 256);                     // rotated image
  b += align_up((size_t)(n > 0 ? n : 1) * sizeof(float), 256) * 3;      // f, s, coef
  b += align_up((size_t)p.chunks * p.ldp * sizeof(float), 256);          // partials
  p.ws_bytes = b + 256;
  return p;
}

template <bool MAT, typename TE, typename TC>
static void launch_sparse_weight(const SpRows<TC>& rows, int64_t n, int64_t vf, const float* x, const TE* eff,
                                 int64_t ld_eff, const UpTaps& taps, float* f, float* s, float* coef, float* part,
                                 const SpPlan& p, cudaStream_t st) {
  constexpr int EB = 8;
  JSCC_TIMED("sparse_forward", st,
             (sparse_forward_kernel<EB, MAT, TE, TC><<<(unsigned)((n + EB - 1) / EB), kSpThreads, 0, st>>>(
                 rows, n, vf, x, eff, ld_eff, taps, f, s)));
  launch_counter().fetch_add(1);
  int64_t cb = (n + 255) / 256;
  if (cb > 4096) cb = 4096;
  JSCC_TIMED("sparse_coef", st, (sparse_coef_kernel<MAT><<<(unsigned)cb, 256, 0, st>>>(f, s, n, coef)));
  launch_counter().fetch_add(1);
  dim3 bgrid((unsigned)((vf + kSpThreads - 1) / kSpThreads), (unsigned)p.chunks);
  JSCC_TIMED("sparse_back", st,
             (sparse_back_kernel<MAT, TE, TC><<<bgrid, kSpThreads, 0, st>>>(rows, n, p.ev_per_chunk, vf, coef, eff,
                                                                            ld_eff, taps, part, p.ldp)));
  launch_counter().fetch_add(1);
}

template <typename TC>
static int sparse_weight_impl(const SpRows<TC>& rows, int64_t n_events, const void* sysmat, int32_t sysmat_dtype,
                              int64_t ld_sysmat, const UpTaps& t, int64_t vf, int32_t mode, const float* img,
                              const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, float scale,
                              float* weight, void* workspace, size_t workspace_bytes, cudaStream_t st) {
  const SpPlan p = plan_sparse(n_events, vf);
  JSCC_REQUIRE(workspace && workspace_bytes >= p.ws_bytes, "jscc_sparse_weight: workspace too small (%zu < %zu)",
               workspace_bytes, p.ws_bytes);
  Carver cv(workspace, workspace_bytes);
  float* xr = cv.take<float>((size_t)p.ldp);
  float* f = cv.take<float>((size_t)n_events);
  float* s = cv.take<float>((size_t)n_events);
  float* coef = cv.take<float>((size_t)n_events);
  float* part = cv.take<float>((size_t)p.chunks * p.ldp);
  JSCC_REQUIRE(cv.ok(), "jscc_sparse_weight: workspace carve overflow");
  const float* x = img;
  if (rotmat) {
    int64_t blocks = (vf + 255) / 256;
    if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
    JSCC_TIMED("sc_gather_rot", st,
               (sc_gather_rot_kernel<<<(unsigned)blocks, 256, 0, st>>>(img, rotmat, ld_rot, 0, 1, vf, p.ldp, xr)));
    JSCC_LAUNCH_CHECK();
    x = xr;
  }
  const bool mat = mode == JSCC_SPARSE_MATERIALIZE;
  if (sysmat_dtype == JSCC_DTYPE_F32) {
    const float* e = static_cast<const float*>(sysmat);
    if (mat) launch_sparse_weight<true, float, TC>(rows, n_events, vf, x, e, ld_sysmat, t, f, s, coef, part, p, st);
    else launch_sparse_weight<false, float, TC>(rows, n_events, vf, x, e, ld_sysmat, t, f, s, coef, part, p, st);
  } else {
    const __nv_bfloat16* e = static_cast<const __nv_bfloat16*>(sysmat);
    if (mat)
      launch_sparse_weight<true, __nv_bfloat16, TC>(rows, n_events, vf, x, e, ld_sysmat, t, f, s, coef, part, p, st);
    else
      launch_sparse_weight<false, __nv_bfloat16, TC>(rows, n_events, vf, x, e, ld_sysmat, t, f, s, coef, part, p, st);
  }
  JSCC_CUDA_CHECK(cudaGetLastError());
  int64_t blocks = (vf + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  const int has_scale = scale != 1.0f;
  JSCC_TIMED("sparse_reduce", st,
             (sparse_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part, p.ldp, (int)p.chunks, rotmat_inv, ld_rot, vf,
                                                                     has_scale, scale, weight)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

// ------------------------------------------------------------------ grouped coarse-space weight
// Events sharing a first-hit row g share that sysmat row, so with v_ij = up(t_i)[j] A[g, j]:
//   f_i = sum_j v_ij x_j = t_i . adj(A_g * x)          (adjoint of the upsample, coarse grid)
//   S_i = sum_j v_ij     = t_i . adj(A_g)              (fixed per event: computed once)
//   w_j += sum_i v_ij c_i = A[g, j] * up(q_g)[j],  q_g = sum_{i in g} c_i t_i
// Two kernels, both deterministic:
//   group_coef:    one CTA per group (grid-stride): adj(A_g * x) in shared memory, per-event
//                  coarse dots -> c_i, then q_g written to the workspace;
//   group_scatter: one thread per fine voxel (its taps in registers) x a chunk of groups,
//                  partial sums per chunk, reduced in chunk order by sparse_reduce.
// Events are visited through `order` (event indices sorted by row).

constexpr int kGcThreads = 256;

// xw[k][c] = w[k][c] * x[j[k][c]] : the adjoint taps with the image folded in (once per call)
__global__ void sparse_fold_x_kernel(const int32_t* __restrict__ tj, const float* __restrict__ tw, int64_t n,
                                     const float* __restrict__ x, float* __restrict__ xw) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    xw[t] = tw[t] * __ldg(x + tj[t]);
}

// The adjoint taps packed in pairs for the bulk pipeline: tp[m][c] = (j[2m][c], w'[2m][c],
// j[2m+1][c], w'[2m+1][c]) with w' = w * x[j] (x null: w' = w), m < ceil(K / 2); a tap
// past K is (0, 0). One 16-byte load brings two taps.
__global__ void sparse_fold_pack_kernel(const int32_t* __restrict__ tj, const float* __restrict__ tw, int K, int M,
                                        int64_t vc, const float* __restrict__ x, int4* __restrict__ tp) {
  const int64_t n = (int64_t)M * vc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / vc);
    const int64_t c = t - (int64_t)m * vc;
    int idx[2] = {0, 0};
    float w[2] = {0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 2 * m + h;
      if (k < K) {
        idx[h] = tj[(int64_t)k * vc + c];
        w[h] = x ? tw[(int64_t)k * vc + c] * __ldg(x + idx[h]) : tw[(int64_t)k * vc + c];
      }
    }
    tp[t] = make_int4(idx[0], __float_as_int(w[0]), idx[1], __float_as_int(w[1]));
  }
}

// The adjoint of a ring stencil of stride 4 (lateral theta interpolation with stride 4 in
// every ring, z the identity; the host checks the tap table has exactly this form): coarse
// c = zc * n_lc + lc, lc = r * n_thc + th, centre jb = zc * n_lf + r * ring_len + 4 th, taps
// jb + d for d = -3..3 (ring-periodic, which only th = 0 needs). xs[c] = the seven folded
// weights w * x[j] (x null: w) in d order and, in the eighth float, jb | (th == 0) << 30.
__global__ void sparse_fold_ring_kernel(const int32_t* __restrict__ tj, const float* __restrict__ tw, int K, int vc,
                                        int n_lc, int n_lf, int ring_len, const float* __restrict__ x,
                                        float4* __restrict__ xs) {
  const int n_thc = ring_len / 4;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < vc; c += gridDim.x * blockDim.x) {
    const int zc = c / n_lc, lc = c - zc * n_lc;
    const int r = lc / n_thc, th = lc - r * n_thc;
    const int jb = zc * n_lf + r * ring_len + 4 * th;
    float w[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < K; ++k) {
      const int j = tj[(int64_t)k * vc + c];
      int d = j - jb;
      if (d > 3) d -= ring_len;
      if (d < -3) d += ring_len;
      if (d >= -3 && d <= 3) w[d + 3] = x ? tw[(int64_t)k * vc + c] * __ldg(x + j) : tw[(int64_t)k * vc + c];
    }
    xs[2 * c] = make_float4(w[0], w[1], w[2], w[3]);
    xs[2 * c + 1] = make_float4(w[4], w[5], w[6], __int_as_float(jb | (th == 0 ? 1 << 30 : 0)));
  }
}

// Dot of a coarse row (global, TC) with a shared-memory vector, by one warp; 16-byte loads
// with four independent accumulators when the row is 16-byte aligned.
template <typename TC>
__device__ __forceinline__ float warp_row_dot(const TC* __restrict__ tc, const float* b, int64_t vc, bool vec,
                                              int lane) {
  constexpr int NV = 16 / (int)sizeof(TC);
  float f0 = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f;
  int64_t tail = 0;
  if (vec) {
    const int64_t nv = vc / NV;
    tail = nv * NV;
#pragma unroll 4
    for (int64_t v = lane; v < nv; v += 32) {
      const uint4 raw = __ldg(reinterpret_cast<const uint4*>(tc) + v);
      const float* bb = b + v * NV;
      if (sizeof(TC) == 2) {
        f0 = fmaf(bf16_lo(raw.x), bb[0], f0);
        f1 = fmaf(bf16_hi(raw.x), bb[1], f1);
        f2 = fmaf(bf16_lo(raw.y), bb[2], f2);
        f3 = fmaf(bf16_hi(raw.y), bb[3], f3);
        f0 = fmaf(bf16_lo(raw.z), bb[4], f0);
        f1 = fmaf(bf16_hi(raw.z), bb[5], f1);
        f2 = fmaf(bf16_lo(raw.w), bb[6], f2);
        f3 = fmaf(bf16_hi(raw.w), bb[7], f3);
      } else {
        f0 = fmaf(__uint_as_float(raw.x), bb[0], f0);
        f1 = fmaf(__uint_as_float(raw.y), bb[1], f1);
        f2 = fmaf(__uint_as_float(raw.z), bb[2], f2);
        f3 = fmaf(__uint_as_float(raw.w), bb[3], f3);
      }
    }
  }
  for (int64_t c = tail + lane; c < vc; c += 32) f0 = fmaf(ld_any(tc, c), b[c], f0);
  return warp_sum((f0 + f1) + (f2 + f3));
}

// MODE 0: materialise semantics (reads S), 1: grouped semantics, 2: compute S (adjoint of A_g
// alone, no q). Adjoint taps: fixed width K, tj/tw(or xw) [K][vc] (padding has weight 0).
// Adjoint of one group: b[c] = sum_k tw[k][c] * A_g[tj[k][c]], four coarse voxels per thread
// at a time; with a compile-time width KT all index loads, then all gathers, are issued
// before the first FMA (KT = 0: runtime width K).
template <int KT, typename TE>
__device__ __forceinline__ void group_adjoint(float* b, int64_t vc, const int32_t* __restrict__ tj,
                                              const float* __restrict__ tw, int K, const TE* __restrict__ er,
                                              int tid) {
  for (int64_t c0 = tid; c0 < vc; c0 += 4 * kGcThreads) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if (KT > 0) {
      int idx[4][KT > 0 ? KT : 1];
      float wv[4][KT > 0 ? KT : 1];
#pragma unroll
      for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t c = c0 + (int64_t)u * kGcThreads;
          const bool in = c < vc && k < K;  // the table has K rows; KT may exceed K
          idx[u][k] = in ? __ldg(tj + (int64_t)k * vc + c) : 0;
          wv[u][k] = in ? __ldg(tw + (int64_t)k * vc + c) : 0.f;
        }
      float av[4][KT > 0 ? KT : 1];
#pragma unroll
      for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int u = 0; u < 4; ++u) av[u][k] = ld_any(er, idx[u][k]);
#pragma unroll
      for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fmaf(wv[u][k], av[u][k], acc[u]);
    } else {
      for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t c = c0 + (int64_t)u * kGcThreads;
          if (c < vc) {
            const float wvv = __ldg(tw + (int64_t)k * vc + c);
            if (wvv != 0.f) acc[u] = fmaf(wvv, ld_any(er, __ldg(tj + (int64_t)k * vc + c)), acc[u]);
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t c = c0 + (int64_t)u * kGcThreads;
      if (c < vc) b[c] = acc[u];
    }
  }
}

// four consecutive coarse values of a row (8-byte loads for bf16, 16-byte for float when aligned)
template <typename TC>
__device__ __forceinline__ void load4(const TC* p, int64_t c, bool vec, float (&v)[4]);
template <>
__device__ __forceinline__ void load4<__nv_bfloat16>(const __nv_bfloat16* p, int64_t c, bool vec, float (&v)[4]) {
  if (vec) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(p + c));
    v[0] = bf16_lo(u.x); v[1] = bf16_hi(u.x); v[2] = bf16_lo(u.y); v[3] = bf16_hi(u.y);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __bfloat162float(p[c + k]);
  }
}
template <>
__device__ __forceinline__ void load4<float>(const float* p, int64_t c, bool vec, float (&v)[4]) {
  if (vec) {
    const float4 u = __ldg(reinterpret_cast<const float4*>(p + c));
    v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __ldg(p + c + k);
  }
}

template <int MODE, int KT, typename TE, typename TC>
__global__ void __launch_bounds__(kGcThreads)
sparse_group_coef_kernel(SpRows<TC> rows, bool vec_rows, const int32_t* __restrict__ order,
                         const int32_t* __restrict__ goff, const int32_t* __restrict__ grow, int n_groups, int64_t vc,
                         const int32_t* __restrict__ tj, const float* __restrict__ tw, int K,
                         const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ s_ev, float* __restrict__ coef,
                         float* __restrict__ q, int64_t ldq) {
  extern __shared__ float4 sm4[];
  float* b = reinterpret_cast<float*>(sm4);  // [vc]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NVq = 4;  // coarse values per thread-slot in the q pass
  for (int gi = blockIdx.x; gi < n_groups; gi += gridDim.x) {
    const TE* er = eff + clamp_row(grow[gi], rows.n_det) * ld_eff;
    const int e0 = goff[gi], e1 = goff[gi + 1];
    __syncthreads();
    // b[c] = sum_k tw[k][c] * A_g[tj[k][c]]  (x already folded into tw except for MODE 2)
    group_adjoint<KT, TE>(b, vc, tj, tw, K, er, tid);
    __syncthreads();
    for (int e = e0 + warp; e < e1; e += kGcThreads / 32) {
      const int64_t i = order[e];
      const float f = warp_row_dot<TC>(rows.coarse(i), b, vc, vec_rows, lane);
      if (lane == 0) {
        if (MODE == 2) {
          s_ev[e] = f;  // event sums are kept by position in `order`
        } else if (MODE == 0) {
          const float si = s_ev[e];
          coef[i] = (isfinite(si) && si > 0.f) ? (1.0f / fmaxf(f / si, 1e-12f)) / si : 0.f;
        } else {
          coef[i] = 1.0f / fmaxf(f, 1e-12f);
        }
      }
    }
    if (MODE == 2) continue;
    __syncthreads();
    // q_g = sum_i c_i t_i : each thread owns 4 consecutive coarse values; events in order
    float* qg = q + (int64_t)gi * ldq;
    const bool vq = vec_rows && (vc % 4 == 0);
    for (int64_t c0 = (int64_t)tid * NVq; c0 < vc; c0 += (int64_t)kGcThreads * NVq) {
      float acc[NVq] = {0.f, 0.f, 0.f, 0.f};
      const bool full = c0 + NVq <= vc;
      for (int e = e0; e < e1; ++e) {
        const int64_t i = order[e];
        const float ci = coef[i];
        if (ci == 0.f) continue;
        const TC* tc = rows.coarse(i);
        if (full) {
          float v[4];
          load4<TC>(tc, c0, vq, v);
#pragma unroll
          for (int u = 0; u < NVq; ++u) acc[u] = fmaf(ci, v[u], acc[u]);
        } else {
          for (int u = 0; u < NVq; ++u)
            if (c0 + u < vc) acc[u] = fmaf(ci, ld_any(tc, c0 + u), acc[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < NVq; ++u)
        if (c0 + u < vc) qg[c0 + u] = acc[u];
    }
  }
}

// ------------------------------------------------------------------ grouped coefficients, bulk-copy pipeline
// The per-group computation in two kernels whose operands move by bulk copies
// (cp.async.bulk completing on mbarriers), each byte read from HBM once:
//   sparse_group_adjoint: b_g = adjoint of (A_g o x) for every group into `bq` (float,
//     [n_groups][ldq]). For the stride-4 ring stencil a CTA takes one tile of whole rings and
//     one chunk of the groups: its threads keep the tile's folded taps (x folded in) in
//     registers for the whole chunk while thread 0 streams the groups' sysmat-row segments
//     through a ring of shared-memory stages, so the taps are read once per CTA rather than
//     once per group. Other tap tables: one thread per coarse voxel gathering the sysmat row
//     from global memory.
//   sparse_group_coef (this kernel): one persistent CTA per SM walks its groups
//     gi = blockIdx.x, + gridDim.x, ... (group k of the CTA) with two warp roles:
//     producer (warp 15): b_g into one shared buffer (once the event warps have taken the
//       previous group's b into registers) and every event's coarse row, in order, into a
//       ring of `n_slots` slots;
//     event warps (0-14): each thread holds b and q of its coarse values c = 4 t + 1,920 u in
//       registers for the group; chunks of up to `batch` events: dots f_i = t_i . b (per
//       thread, then per warp, then over warps in warp order after one named barrier),
//       coefficients, q += c_i t_i (events in order); q_g stored at the end of the group.
// Shared memory: header (barriers, flags, dot partials), b[vc] float, slots[n_slots][vc] TC.
// Every wait is bounded: on a timeout the CTA counts it (jscc_take_wait_timeout_count),
// waits (bounded) for the copies it still has in flight and returns.
constexpr int kBkThreads = 512;
constexpr int kBkEventWarps = 15;
constexpr int kBkEvents = kBkEventWarps * 32;
constexpr int kBkProducerWarp = kBkEventWarps;
constexpr int kBkMaxSlots = 16;
constexpr int kBkMaxBatch = 4;  // events of a chunk
constexpr int kBkQ = 5;         // b and q registers: chunks of four coarse values per event thread
constexpr int64_t kBkMaxCoarse = (int64_t)kBkQ * 4 * kBkEvents;
constexpr int kBkHeader = 1024;  // barriers, flags, dot partials
constexpr uint32_t kBkMaxPolls = 1u << 22;    // default bound of a pipeline wait
constexpr uint32_t kBkDrainPolls = 1u << 24;  // bound of the drain of a CTA that gave up
static_assert(kBkProducerWarp * 32 + 32 == kBkThreads, "warp roles");
static_assert(2 * kBkMaxSlots * 8 + 64 + 2 * kBkEventWarps * kBkMaxBatch * 4 <= kBkHeader, "header");

__device__ unsigned int g_wait_timeout_count = 0;
// Poll bound of the pipeline waits of the bulk kernels, settable from the host
// (jscc_set_wait_limit): 0 makes every such wait give up at once, which exercises the
// give-up path while every copy still completes. The drains keep their own fixed bound.
__device__ uint32_t g_bk_poll_limit = kBkMaxPolls;

// acc.xyzw += v[0..3] * b.xyzw as two packed f32x2 FMAs: per lane the same round-to-nearest FMA
// as fmaf, in half the issued instructions
__device__ __forceinline__ void ffma4(float4& acc, const float (&v)[4], const float4& b) {
  const float2 lo = __ffma2_rn(make_float2(v[0], v[1]), make_float2(b.x, b.y), make_float2(acc.x, acc.y));
  const float2 hi = __ffma2_rn(make_float2(v[2], v[3]), make_float2(b.z, b.w), make_float2(acc.z, acc.w));
  acc = make_float4(lo.x, lo.y, hi.x, hi.y);
}
// acc.xyzw += c * v[0..3] (packed, as ffma4)
__device__ __forceinline__ void ffma4s(float4& acc, float c, const float (&v)[4]) {
  const float2 cc = make_float2(c, c);
  const float2 lo = __ffma2_rn(cc, make_float2(v[0], v[1]), make_float2(acc.x, acc.y));
  const float2 hi = __ffma2_rn(cc, make_float2(v[2], v[3]), make_float2(acc.z, acc.w));
  acc = make_float4(lo.x, lo.y, hi.x, hi.y);
}

// four consecutive coarse values from shared memory (c a multiple of 4)
__device__ __forceinline__ void smem4(const __nv_bfloat16* p, int64_t c, float (&v)[4]) {
  const uint2 u = *reinterpret_cast<const uint2*>(p + c);
  v[0] = bf16_lo(u.x); v[1] = bf16_hi(u.x); v[2] = bf16_lo(u.y); v[3] = bf16_hi(u.y);
}
__device__ __forceinline__ void smem4(const float* p, int64_t c, float (&v)[4]) {
  const float4 u = *reinterpret_cast<const float4*>(p + c);
  v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
}

// two runs of four consecutive values at p and p + 128 (plain loads; p 8-byte aligned for
// BF16, 16-byte aligned for float)
template <typename T>
__device__ __forceinline__ void load4x2(const T* p, float (&v)[8]) {
  float a[4], b[4];
  smem4(p, 0, a);
  smem4(p + 128, 0, b);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[i] = a[i];
    v[4 + i] = b[i];
  }
}

// ---- sparse_group_adjoint, stride-4 ring stencil
constexpr int kAdWarps = 8;  // compute warps; one more warp streams the segments
constexpr int kAdThreads = kAdWarps * 32 + 32;
constexpr int kAdCompute = kAdWarps * 32;
constexpr int kAdVox = 4;  // coarse voxels per compute thread: a tile holds at most 1,024
constexpr int kAdMaxStages = 8;
constexpr int kAdHeader = 256;

// Coarse voxel c of the tile [c0, c1) (whole rings: a voxel at theta 0 takes its taps
// d = -3..-1 from the end of its own ring, inside the tile): taps xs[c] (x folded in) and, in
// the eighth float, jb | (th == 0) << 30 with jb = 4 c. b[c] = sum_{d=-3..3} xs[c][d] *
// seg[jb - 4 c0 + d], the taps in d order as one packed f32x2 chain per pair of voxels (the
// same fmaf sequence per lane). The producer warp issues group k + n_stages's segment into a
// stage once every compute warp has released it (empty[s], one arrival per warp).
template <typename TE>
__global__ void __launch_bounds__(kAdThreads)
sparse_group_adjoint_ring_kernel(const int32_t* __restrict__ grow, int n_groups, int gpc, const TE* __restrict__ eff,
                                 int64_t ld_eff, int64_t n_det, const float4* __restrict__ xs, int vc, int tile_c,
                                 int ring_len, float* __restrict__ bq, int64_t ldq, int n_stages,
                                 uint32_t stage_stride) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kAdMaxStages]
  uint64_t* empty = full + kAdMaxStages;                // [kAdMaxStages]
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 2 * kAdMaxStages * 8);
  int* issued = reinterpret_cast<int*>(smem + 2 * kAdMaxStages * 8 + 4);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c0 = blockIdx.x * tile_c, c1 = min(vc, c0 + tile_c);
  const int g0 = blockIdx.y * gpc, g1 = min(n_groups, g0 + gpc);
  if (c0 >= c1 || g0 >= g1) return;
  const uint32_t seg_bytes = (uint32_t)(c1 - c0) * 4u * (uint32_t)sizeof(TE);
  auto stage = [&](int s) { return reinterpret_cast<const TE*>(smem + kAdHeader + (size_t)s * stage_stride); };
  const uint32_t polls = g_bk_poll_limit;
  const int n_k = g1 - g0;
  if (tid == 0) {
    for (int s = 0; s < kAdMaxStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, kAdWarps);
    }
    *abort_flag = 0;
    *issued = 0;
    mbar_init_fence();
  }
  __syncthreads();
  if (warp == kAdWarps) {
    // ---- producer: segment of group k into stage k mod n_stages; 32 row indices per window
    int win_base = INT_MIN, win_val = 0;
    for (int k = 0; k < n_k; ++k) {
      const int s = k % n_stages;
      bool ok = k < n_stages || bk_wait(empty + s, (uint32_t)(k / n_stages - 1) & 1u, abort_flag, polls);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      if (k >= win_base + 32 || win_base == INT_MIN) {
        win_base = k;
        win_val = k + lane < n_k ? grow[g0 + k + lane] : 0;
      }
      const int row = __shfl_sync(0xffffffffu, win_val, k - win_base);
      if (lane == 0) {
        mbar_arrive_expect_tx(full + s, seg_bytes);
        bulk_copy_g2s(const_cast<TE*>(stage(s)), eff + clamp_row(row, n_det) * ld_eff + 4 * (int64_t)c0, seg_bytes,
                      full + s);
        *issued = k + 1;
      }
    }
  } else {
    // ---- compute warps: the tile's taps in registers, one group per stage
    float4 wa[kAdVox], wb[kAdVox];
#pragma unroll
    for (int u = 0; u < kAdVox; ++u) {
      const int c = c0 + tid + u * kAdCompute;
      wa[u] = c < c1 ? __ldg(xs + 2 * c) : make_float4(0.f, 0.f, 0.f, 0.f);
      wb[u] = c < c1 ? __ldg(xs + 2 * c + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int k = 0; k < n_k; ++k) {
      const int s = k % n_stages;
      bool ok = bk_wait(full + s, (uint32_t)(k / n_stages) & 1u, abort_flag, polls);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      const TE* seg = stage(s);
      float* out = bq + (int64_t)(g0 + k) * ldq;
#pragma unroll
      for (int u = 0; u < kAdVox; u += 2) {
        float v[2][8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int c = c0 + tid + (u + h) * kAdCompute;
          if (c < c1) {
            const int info = __float_as_int(wb[u + h].w);
            const int jl = (info & 0x3fffffff) - 4 * c0;  // centre within the segment
            float a4[4], b4[4];
            smem4(seg + ((info >> 30) ? jl - 4 + ring_len : jl - 4), 0, a4);
            smem4(seg + jl, 0, b4);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              v[h][i] = a4[i];
              v[h][4 + i] = b4[i];
            }
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) v[h][i] = 0.f;
          }
        }
        const float w0[7] = {wa[u].x, wa[u].y, wa[u].z, wa[u].w, wb[u].x, wb[u].y, wb[u].z};
        const float w1[7] = {wa[u + 1].x, wa[u + 1].y, wa[u + 1].z, wa[u + 1].w, wb[u + 1].x, wb[u + 1].y,
                             wb[u + 1].z};
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int d = 0; d < 7; ++d)
          acc = __ffma2_rn(make_float2(w0[d], w1[d]), make_float2(v[0][d + 1], v[1][d + 1]), acc);
        const int ca = c0 + tid + u * kAdCompute, cb = ca + kAdCompute;
        if (ca < c1) out[ca] = acc.x;
        if (cb < c1) out[cb] = acc.y;
      }
      __syncwarp();  // every lane is past its reads of stage s
      if (lane == 0) mbar_arrive(empty + s);
    }
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    // copies still in flight write this CTA's shared memory: wait (bounded) for them
    for (int k = max(0, *issued - n_stages); k < *issued; ++k)
      mbar_wait_bounded(full + k % n_stages, (uint32_t)(k / n_stages) & 1u, kBkDrainPolls);
  }
}

// ---- sparse_group_adjoint, packed tap table (any upsample): b[c] = sum over the packed
// taps (index, w x) of w' * A_g[j], one thread per coarse voxel, the sysmat row gathered
// from global memory (cached); with MT = KT / 2 > 0 all tap loads are issued first.
template <int KT, typename TE>
__global__ void __launch_bounds__(256)
sparse_group_adjoint_taps_kernel(const int32_t* __restrict__ grow, int n_groups, const TE* __restrict__ eff,
                                 int64_t ld_eff, int64_t n_det, const int4* __restrict__ tp, int M, int vc,
                                 float* __restrict__ bq, int64_t ldq) {
  constexpr int MT = KT / 2;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= vc) return;
  int4 t[MT > 0 ? MT : 1];
  if (MT > 0) {
#pragma unroll
    for (int m = 0; m < MT; ++m) t[m] = m < M ? __ldg(tp + (size_t)m * vc + c) : make_int4(0, 0, 0, 0);
  }
  for (int g = blockIdx.y; g < n_groups; g += gridDim.y) {
    const TE* er = eff + clamp_row(grow[g], n_det) * ld_eff;
    float acc = 0.f;
    if (MT > 0) {
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        acc = fmaf(__int_as_float(t[m].y), load_elem(er, t[m].x), acc);
        acc = fmaf(__int_as_float(t[m].w), load_elem(er, t[m].z), acc);
      }
    } else {
      for (int m = 0; m < M; ++m) {
        const int4 tt = __ldg(tp + (size_t)m * vc + c);
        acc = fmaf(__int_as_float(tt.y), load_elem(er, tt.x), acc);
        acc = fmaf(__int_as_float(tt.w), load_elem(er, tt.z), acc);
      }
    }
    bq[(int64_t)g * ldq + c] = acc;
  }
}

// ---- sparse_group_coef (bulk): MODE 0 materialise coefficients, 1 grouped, 2 event sums;
// RAGGED: vc is not a multiple of four, so the last four-value chunk is masked
template <int MODE, typename TC, bool RAGGED>
__global__ void __launch_bounds__(kBkThreads, 1)
sparse_group_coef_bulk_kernel(SpRows<TC> rows, const int32_t* __restrict__ order, const int32_t* __restrict__ goff,
                              int n_groups, int vc, const float* __restrict__ bq, float* __restrict__ s_ev,
                              float* __restrict__ q, int64_t ldq, int n_slots, int batch, uint32_t b_bytes,
                              uint32_t row_bytes, uint32_t slot_off, uint32_t slot_stride) {
  constexpr int MB = kBkMaxBatch;  // events of a chunk at most
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kBkMaxSlots]
  uint64_t* empty = full + kBkMaxSlots;                // [kBkMaxSlots]
  uint64_t* b_full = empty + kBkMaxSlots;
  uint64_t* b_empty = b_full + 1;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 2 * kBkMaxSlots * 8 + 16);
  int* rows_issued = reinterpret_cast<int*>(smem + 2 * kBkMaxSlots * 8 + 20);
  int* b_issued = reinterpret_cast<int*>(smem + 2 * kBkMaxSlots * 8 + 24);
  int* rows_used = reinterpret_cast<int*>(smem + 2 * kBkMaxSlots * 8 + 28);
  int* b_used = reinterpret_cast<int*>(smem + 2 * kBkMaxSlots * 8 + 32);
  float* red = reinterpret_cast<float*>(smem + 2 * kBkMaxSlots * 8 + 64);  // [2][kBkEventWarps][kBkMaxBatch]
  float* b = reinterpret_cast<float*>(smem + kBkHeader);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t polls = g_bk_poll_limit;
  const int G = gridDim.x;
  auto slot = [&](int s) { return reinterpret_cast<const TC*>(smem + slot_off + (size_t)s * slot_stride); };
  if (tid == 0) {
    for (int s = 0; s < kBkMaxSlots; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, kBkEventWarps);  // every event warp releases a slot after its reads
    }
    mbar_init(b_full, 1);
    mbar_init(b_empty, kBkEventWarps);
    *abort_flag = 0;
    *rows_issued = *b_issued = *rows_used = *b_used = 0;
    mbar_init_fence();
  }
  __syncthreads();
  if (warp == kBkProducerWarp) {
    // ------------------------------------------------------------ producer warp
    // b stream: group bg (k-th of the CTA: bk); row stream: event re of group rg
    int bg = blockIdx.x, bk = 0;
    int rg = blockIdx.x, re = 0, re_end = 0, pseq = 0;
    if (rg < n_groups) {
      re = goff[rg];
      re_end = goff[rg + 1];
    }
    int win_base = INT_MIN, win_val = 0;  // 32 order values, one per lane
    int ps = 0;            // slot of row pseq (pseq mod n_slots, kept incrementally)
    uint32_t uses = 0;     // bit s: parity of the number of rows issued into slot s
    uint32_t idle = 0;
    bool ok = true;
    while (ok) {
      while (rg < n_groups && re >= re_end) {  // next group with events
        rg += G;
        if (rg < n_groups) {
          re = goff[rg];
          re_end = goff[rg + 1];
          win_base = INT_MIN;  // the window holds one group's events only
        }
      }
      const bool rows_left = rg < n_groups, b_left = bg < n_groups;
      if (!rows_left && !b_left) break;
      bool progress = false;
      if (b_left) {
        // the event warps have taken group bk - 1's b into registers: phase bk - 1 of b_empty
        bool ready = bk == 0 || mbar_test_wait(b_empty, (bk - 1) & 1);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          if (lane == 0) {
            mbar_arrive_expect_tx(b_full, b_bytes);
            bulk_copy_g2s(b, bq + (int64_t)bg * ldq, b_bytes, b_full);
            *b_issued = bk + 1;
          }
          bg += G;
          ++bk;
          progress = true;
        }
      }
      if (rows_left) {
        const int s = ps;
        // the slot's previous row (use u - 1) must have been released: phase u - 1 of empty[s]
        bool ready = pseq < n_slots || mbar_test_wait(empty + s, ((uses >> s) & 1u) ^ 1u);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          if (re < win_base || re >= win_base + 32) {  // refill the window of event indices
            win_base = re;
            win_val = re + lane < re_end ? order[re + lane] : 0;
          }
          const int i = __shfl_sync(0xffffffffu, win_val, re - win_base);
          if (lane == 0) {
            mbar_arrive_expect_tx(full + s, row_bytes);
            bulk_copy_g2s(const_cast<TC*>(slot(s)), rows.coarse(i), row_bytes, full + s);
            *rows_issued = pseq + 1;
          }
          uses ^= 1u << s;
          ps = ps + 1 == n_slots ? 0 : ps + 1;
          ++pseq;
          ++re;
          progress = true;
        }
      }
      if (progress) {
        idle = 0;
      } else if (++idle > polls || *abort_flag) {
        ok = false;
      } else {
        __nanosleep(64);  // neither buffer is free yet: leave the issue slots to the other warps
      }
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else {
    // ------------------------------------------------------------ event warps
    const int et = tid;
    int seq = 0, kg = 0, par = 0;
    int cs_slot = 0;         // slot of event seq (seq mod n_slots, kept incrementally)
    uint32_t cphase = 0;     // bit s: parity of the next phase of full[s]
    bool aborted = false, bad = false;  // bad: one of this thread's waits gave up
    // the event ranges of the next two groups are loaded while a group is processed
    auto range = [&](int g, int& a, int& e) {
      a = g < n_groups ? goff[g] : 0;
      e = g < n_groups ? goff[g + 1] : 0;
    };
    int r0a, r0e, r1a, r1e;
    range(blockIdx.x, r0a, r0e);
    range(blockIdx.x + G, r1a, r1e);
    for (int gi = blockIdx.x; gi < n_groups && !aborted; gi += G, ++kg) {
      const int e0 = r0a, e1 = r0e;
      r0a = r1a;
      r0e = r1e;
      range(gi + 2 * G, r1a, r1e);
      // b of this thread's coarse values into registers, then the buffer goes back
      if (!bk_wait(b_full, kg & 1, abort_flag, polls)) bad = true;
      float4 bv[kBkQ], qa[kBkQ];
#pragma unroll
      for (int u = 0; u < kBkQ; ++u) {
        const int c = et * 4 + u * (kBkEvents * 4);
        bv[u] = c < vc ? *reinterpret_cast<const float4*>(b + c) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (RAGGED && c < vc && c + 4 > vc) {  // the tail past vc is padding
          if (c + 1 >= vc) bv[u].y = 0.f;
          if (c + 2 >= vc) bv[u].z = 0.f;
          bv[u].w = 0.f;
        }
        qa[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      __syncwarp();
      if (__all_sync(0xffffffffu, !bad) && lane == 0) {
        if (et == 0) *b_used = kg + 1;
        mbar_arrive(b_empty);
      }
      // one chunk of NE events, NE known when compiled (no issue slots for absent events);
      // false: one of the waits gave up
      auto chunk = [&](auto ne_tag, int bs) -> bool {
        constexpr int NE = decltype(ne_tag)::value;
        // the event sum of lane k's event of the chunk, read before the dots
        const float s_lane = (MODE == 0 && lane < NE) ? s_ev[bs + lane] : 0.f;
        int sl[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
          sl[k] = cs_slot;
          cs_slot = cs_slot + 1 == n_slots ? 0 : cs_slot + 1;
        }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
          if (!bk_wait(full + sl[k], (cphase >> sl[k]) & 1u, abort_flag, polls)) bad = true;
          cphase ^= 1u << sl[k];
        }
        // ---- dots f_i = t_i . b: this thread's values, then the warp's
        float4 acc[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kBkQ; ++u) {
          const int c = et * 4 + u * (kBkEvents * 4);
          if (c < vc) {
#pragma unroll
            for (int k = 0; k < NE; ++k) {
              float v[4];
              smem4(slot(sl[k]), c, v);
              if (RAGGED && c + 4 > vc) {  // padding past the row (any value) must not reach the dot
#pragma unroll
                for (int e = 1; e < 4; ++e)
                  if (c + e >= vc) v[e] = 0.f;
              }
              ffma4(acc[k], v, bv[u]);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
          const float f = warp_sum((acc[k].x + acc[k].y) + (acc[k].z + acc[k].w));
          if (lane == 0) red[(par * kBkEventWarps + warp) * kBkMaxBatch + k] = f;
        }
        if (role_sync_or(1, kBkEvents, bad)) return false;
        // ---- coefficients: lane k sums event k's partials over the warps in order (every
        // warp the same values), then broadcasts
        float cl = 0.f;
        if (lane < NE) {
          float f = 0.f;
#pragma unroll
          for (int w = 0; w < kBkEventWarps; ++w) f += red[(par * kBkEventWarps + w) * kBkMaxBatch + lane];
          if (MODE == 2) {
            if (warp == 0) s_ev[bs + lane] = f;  // event sums are kept by position in `order`
          } else if (MODE == 0) {
            // (1 / max(f / S, 1e-12)) / S = 1 / max(f, 1e-12 S) for S > 0: one division
            cl = (isfinite(s_lane) && s_lane > 0.f) ? 1.0f / fmaxf(f, 1e-12f * s_lane) : 0.f;
          } else {
            cl = 1.0f / fmaxf(f, 1e-12f);
          }
        }
        // ---- q_g += c_i t_i over the chunk, events in order
        if (MODE != 2) {
#pragma unroll
          for (int k = 0; k < NE; ++k) {
            const float ck = __shfl_sync(0xffffffffu, cl, k);
            if (ck != 0.f) {
#pragma unroll
              for (int u = 0; u < kBkQ; ++u) {
                const int c = et * 4 + u * (kBkEvents * 4);
                if (c < vc) {
                  float v[4];
                  smem4(slot(sl[k]), c, v);
                  ffma4s(qa[u], ck, v);
                }
              }
            }
          }
        }
        // ---- this warp is past its last read of the chunk's rows: release the slots (a
        // warp with a lane whose wait gave up keeps them: its copy may still be in flight)
        __syncwarp();
        if (__all_sync(0xffffffffu, !bad) && lane == 0) {
          if (et == 0) *rows_used = seq + NE;  // before the slots can be refilled
#pragma unroll
          for (int k = 0; k < NE; ++k) mbar_arrive(empty + sl[k]);
        }
        seq += NE;
        par ^= 1;
        return true;
      };
      for (int bs = e0; bs < e1; bs += batch) {
        const int n = min(batch, e1 - bs);
        bool ok;
        if (n == 1) {
          ok = chunk(std::integral_constant<int, 1>{}, bs);
        } else if (n == 2) {
          ok = chunk(std::integral_constant<int, 2>{}, bs);
        } else if (n == 3) {
          ok = chunk(std::integral_constant<int, 3>{}, bs);
        } else {
          ok = chunk(std::integral_constant<int, MB>{}, bs);
        }
        if (!ok) {
          aborted = true;
          break;
        }
      }
      if (aborted) break;
      if (e0 == e1 && role_sync_or(1, kBkEvents, bad)) {  // no chunk consumed the b wait's status
        aborted = true;
        break;
      }
      if (MODE != 2) {
        float* qg = q + (int64_t)gi * ldq;
#pragma unroll
        for (int u = 0; u < kBkQ; ++u) {
          const int c = et * 4 + u * (kBkEvents * 4);
          if (c < vc) *reinterpret_cast<float4*>(qg + c) = qa[u];
        }
      }
    }
    if (aborted) *abort_flag = 1;  // stops the producer
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    // copies still in flight write this CTA's shared memory: wait (bounded) for them
    for (int sq = *rows_used; sq < *rows_issued; ++sq)
      mbar_wait_bounded(full + sq % n_slots, (sq / n_slots) & 1, kBkDrainPolls);
    if (*b_issued > *b_used) mbar_wait_bounded(b_full, *b_used & 1, kBkDrainPolls);
  }
}

// part[chunk][j] = sum_{groups in chunk} A[g, j] * up(q_g)[j]
template <typename TE>
__global__ void __launch_bounds__(256)
sparse_group_scatter_kernel(const float* __restrict__ q, int64_t ldq, const int32_t* __restrict__ grow, int n_groups,
                            int groups_per_chunk, int64_t vf, const TE* __restrict__ eff, int64_t ld_eff,
                            int64_t n_det, UpTaps taps, float* __restrict__ part, int64_t ldp) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= vf) return;
  const int zf = (int)(j / taps.n_lf), lf = (int)(j % taps.n_lf);
  const int l0 = taps.lt[2 * lf], l1 = taps.lt[2 * lf + 1];
  const float w0 = taps.lwt[2 * lf], w1 = taps.lwt[2 * lf + 1];
  const int z0 = taps.zt[2 * zf], z1 = taps.zt[2 * zf + 1];
  const float u0 = taps.zwt[2 * zf], u1 = taps.zwt[2 * zf + 1];
  const int64_t c00 = (int64_t)z0 * taps.n_lc + l0, c01 = (int64_t)z0 * taps.n_lc + l1;
  const int64_t c10 = (int64_t)z1 * taps.n_lc + l0, c11 = (int64_t)z1 * taps.n_lc + l1;
  const int g_begin = blockIdx.y * groups_per_chunk;
  const int g_end = (g_begin + groups_per_chunk) < n_groups ? g_begin + groups_per_chunk : n_groups;
  const bool two_z = u1 != 0.f;
  float acc = 0.f;
  // eight groups at a time: every load of the eight is issued before the first FMA
  constexpr int U = 8;
  for (int g0 = g_begin; g0 < g_end; g0 += U) {
    int64_t off[U];
#pragma unroll
    for (int u = 0; u < U; ++u) off[u] = g0 + u < g_end ? clamp_row(__ldg(grow + g0 + u), n_det) * ld_eff : -1;
    float a[U], p0[U], p1[U], r0[U], r1[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = off[u] >= 0;
      const float* qg = q + (int64_t)(g0 + u) * ldq;
      a[u] = in ? ld_any(eff + off[u], j) : 0.f;
      p0[u] = in ? __ldg(qg + c00) : 0.f;
      p1[u] = in ? __ldg(qg + c01) : 0.f;
      r0[u] = in && two_z ? __ldg(qg + c10) : 0.f;
      r1[u] = in && two_z ? __ldg(qg + c11) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float t = w0 * p0[u];
      t = fmaf(w1, p1[u], t);
      float v = u0 * t;
      if (two_z) {
        float bb = w0 * r0[u];
        bb = fmaf(w1, r1[u], bb);
        v = fmaf(u1, bb, v);
      }
      if (v != 0.f) acc = fmaf(a[u], v, acc);
    }
  }
  part[(int64_t)blockIdx.y * ldp + j] = acc;
}

// Bulk-copy form of the scatter (same arithmetic and group order, so the same result).
// CTA = one tile of kScTile fine voxels of one z plane x one chunk of groups; a producer warp
// streams, per group, the sysmat row's tile and the q segment(s) the tile's lateral taps
// touch ([lmin, lmax] of the tile, one segment per z tap) into a ring of stages; eight
// consumer warps hold their voxels' taps and sums in registers (eight voxels per thread)
// and read only shared memory. A tile whose tap span exceeds a segment reads q and the
// sysmat from global memory instead (no producer). Waits are bounded as in the
// coefficient kernel.
constexpr int kScConsumers = 256;
constexpr int kScThreads = kScConsumers + 32;
constexpr int kScVox = 8;
constexpr int kScTile = kScConsumers * kScVox;
constexpr int kScSeg = 1024;  // coarse values per staged q segment
constexpr int kScMaxStages = 24;
constexpr int kScHeader = 512;  // 2 x kScMaxStages barriers, flags, tap span
static_assert(16 * kScMaxStages + 20 <= kScHeader, "scatter header");

template <typename TE>
__global__ void __launch_bounds__(kScThreads, 2)
sparse_group_scatter_bulk_kernel(const float* __restrict__ q, int64_t ldq, const int32_t* __restrict__ grow,
                                 int n_groups, int groups_per_chunk, const TE* __restrict__ eff, int64_t ld_eff,
                                 int64_t n_det, UpTaps taps, float* __restrict__ part, int64_t ldp,
                                 uint32_t stage_space, uint32_t seg_off) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kScMaxStages]
  uint64_t* empty = full + kScMaxStages;               // [kScMaxStages]
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 16 * kScMaxStages);
  int* issued = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 4);
  int* used = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 8);
  int* span = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 12);  // [lmin, lmax]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t polls = g_bk_poll_limit;
  const int n_lf = taps.n_lf, n_lc = taps.n_lc;
  const int tiles_per_plane = (n_lf + kScTile - 1) / kScTile;
  const int zf = blockIdx.x / tiles_per_plane;
  const int l_begin = (blockIdx.x - zf * tiles_per_plane) * kScTile;
  const int l_end = min(l_begin + kScTile, n_lf);
  const int64_t j0 = (int64_t)zf * n_lf + l_begin;
  const int z0 = taps.zt[2 * zf], z1 = taps.zt[2 * zf + 1];
  const float u0 = taps.zwt[2 * zf], u1 = taps.zwt[2 * zf + 1];
  const bool two_z = u1 != 0.f;
  const int g_begin = blockIdx.y * groups_per_chunk;
  const int g_end = min(g_begin + groups_per_chunk, n_groups);
  if (tid == 0) {
    for (int s = 0; s < kScMaxStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, kScConsumers / 32);
    }
    *abort_flag = 0;
    *issued = *used = 0;
    span[0] = INT_MAX;
    span[1] = -1;
    mbar_init_fence();
  }
  __syncthreads();
  // this thread's voxels and their lateral taps: two runs of four, voxels
  // (warp * 256 + h * 128 + lane * 4 + i), so that one tap of the warp's voxels reads
  // consecutive q words (no bank conflicts) and each run is one 8-byte sysmat load
  const int lf0 = l_begin + warp * (32 * kScVox) + lane * 4;
  auto vox = [&](int v) { return lf0 + (v >> 2) * 128 + (v & 3); };
  int l0[kScVox], l1[kScVox];
  float w0[kScVox], w1[kScVox];
  if (tid < kScConsumers) {
    int mn = INT_MAX, mx = -1;
#pragma unroll
    for (int v = 0; v < kScVox; ++v) {
      const int lf = vox(v);
      const bool in = lf < l_end;
      l0[v] = in ? taps.lt[2 * lf] : 0;
      l1[v] = in ? taps.lt[2 * lf + 1] : 0;
      w0[v] = in ? taps.lwt[2 * lf] : 0.f;
      w1[v] = in ? taps.lwt[2 * lf + 1] : 0.f;
      if (in) {
        mn = min(mn, min(l0[v], l1[v]));
        mx = max(mx, max(l0[v], l1[v]));
      }
    }
    if (mx >= 0) {
      atomicMin(span, mn);
      atomicMax(span + 1, mx);
    }
  }
  __syncthreads();
  const int cs0 = span[0] & ~3;
  const int seg_len = span[1] < 0 ? 4 : ((span[1] + 1 - cs0 + 3) & ~3);
  const bool run1 = lf0 + 128 < l_end;  // the second run of four is in the tile
  if (tid < kScConsumers) {
#pragma unroll
    for (int v = 0; v < kScVox; ++v)
      if (vox(v) >= l_end) l0[v] = l1[v] = cs0;  // (weight 0) keeps every gather inside the segment
  }
  // Two-value runs: when every tap of a run of four voxels is one of two coarse voxels (the
  // polar projector's theta interpolation), the run needs two q loads and each voxel two
  // folded weights, val = ra * q[pc0] + rb * q[pc1]; otherwise the thread gathers each tap.
  int pc0[2], pc1[2];
  float ra[kScVox], rb[kScVox];
  bool pair = true;
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int a = l0[4 * r];
    int b = a;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int v = 4 * r + i;
      if (vox(v) >= l_end) continue;
      const int ls[2] = {l0[v], l1[v]};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (ls[h] == a) continue;
        if (b == a) b = ls[h];
        else if (ls[h] != b) pair = false;
      }
    }
    pc0[r] = a;
    pc1[r] = b;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int v = 4 * r + i;
      const bool in = vox(v) < l_end;
      ra[v] = in ? (l0[v] == a ? w0[v] : 0.f) + (l1[v] == a ? w1[v] : 0.f) : 0.f;
      rb[v] = in && b != a ? (l0[v] == b ? w0[v] : 0.f) + (l1[v] == b ? w1[v] : 0.f) : 0.f;
    }
  }
  // the q segment of z tap t starts at the flat coarse index z_t n_lc + cs0, copied from the
  // 16-byte boundary below it (sh_t values earlier) and clamped to the q row
  const int64_t f0 = (int64_t)z0 * n_lc + cs0, f1 = (int64_t)z1 * n_lc + cs0;
  const int sh0 = (int)(f0 & 3), sh1 = (int)(f1 & 3);
  const int seg_slot = (seg_len + 3 + 3) & ~3;  // a segment and its shift, in whole 16-byte units
  const bool staged = seg_slot <= kScSeg;
  const uint32_t a_bytes = (uint32_t)((l_end - l_begin) * sizeof(TE));
  const uint32_t seg_bytes = (uint32_t)seg_slot * 4u;
  const uint32_t cp0 = (uint32_t)min((int64_t)seg_slot, ldq - (f0 - sh0)) * 4u;
  const uint32_t cp1 = (uint32_t)min((int64_t)seg_slot, ldq - (f1 - sh1)) * 4u;
  // stages sized to this tile's segment: the sysmat tile (seg_off bytes) and one q segment per
  // z tap, as many as the shared memory holds
  const uint32_t stage_bytes = (seg_off + seg_bytes * (two_z ? 2u : 1u) + 127u) & ~127u;
  int n_stages = (int)(stage_space / stage_bytes);
  if (n_stages > kScMaxStages) n_stages = kScMaxStages;
  if (n_stages < 1) n_stages = 1;  // (a tile that is not staged uses none)
  auto stage = [&](int s) { return smem + kScHeader + (size_t)s * stage_bytes; };
  if (warp == kScConsumers / 32) {
    // ------------------------------------------------------------ producer warp
    if (staged) {
      bool ok = true;
      int s = 0;              // stage of group kk (kk mod n_stages, kept incrementally)
      uint32_t eph = 0;       // bit s: parity of the next phase of empty[s] to wait for
      for (int w = g_begin; w < g_end && ok; w += 32) {
        const int gv = w + lane < g_end ? grow[w + lane] : 0;  // 32 group rows per load
        const int m = min(32, g_end - w);
        for (int k = 0; k < m && ok; ++k) {
          const int row = __shfl_sync(0xffffffffu, gv, k);
          const int kk = w - g_begin + k;
          if (lane == 0) {
            if (kk >= n_stages) {
              ok = bk_wait(empty + s, (eph >> s) & 1u, abort_flag, polls);
              eph ^= 1u << s;
            }
            if (ok) {
              unsigned char* st = stage(s);
              const float* qg = q + (int64_t)(w + k) * ldq;
              mbar_arrive_expect_tx(full + s, a_bytes + cp0 + (two_z ? cp1 : 0u));
              bulk_copy_g2s(st, eff + clamp_row(row, n_det) * ld_eff + j0, a_bytes, full + s);
              bulk_copy_g2s(st + seg_off, qg + (f0 - sh0), cp0, full + s);
              if (two_z) bulk_copy_g2s(st + seg_off + seg_bytes, qg + (f1 - sh1), cp1, full + s);
              *issued = kk + 1;
            }
          }
          s = s + 1 == n_stages ? 0 : s + 1;
          ok = __shfl_sync(0xffffffffu, ok, 0);
        }
      }
      if (!ok && lane == 0) *abort_flag = 1;
    }
  } else {
    // ------------------------------------------------------------ consumer warps
    float acc[kScVox];
#pragma unroll
    for (int v = 0; v < kScVox; ++v) acc[v] = 0.f;
    bool bad = false;
    // acc[v] += a[v] * (u0 * (w0 q0[l0] + w1 q0[l1]) + u1 * (w0 q1[l0] + w1 q1[l1]))
    auto accumulate = [&](const float (&a)[kScVox], const float* q0, const float* q1) {
      if (pair && !two_z) {
        // one z plane: per voxel acc += a * (u0 * (ra qa + rb qb)), two voxels per packed f32x2
        // operation (per lane the same rounded operations as the scalar form below)
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const float2 qa = make_float2(q0[pc0[r]], q0[pc0[r]]), qb = make_float2(q0[pc1[r]], q0[pc1[r]]);
#pragma unroll
          for (int i = 0; i < 4; i += 2) {
            const int v = 4 * r + i;
            float2 t = __fmul2_rn(make_float2(ra[v], ra[v + 1]), qa);
            t = __ffma2_rn(make_float2(rb[v], rb[v + 1]), qb, t);
            const float2 val = __fmul2_rn(make_float2(u0, u0), t);
            const float2 nw = __ffma2_rn(make_float2(a[v], a[v + 1]), val, make_float2(acc[v], acc[v + 1]));
            if (val.x != 0.f) acc[v] = nw.x;
            if (val.y != 0.f) acc[v + 1] = nw.y;
          }
        }
        return;
      }
      if (pair) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const float qa = q0[pc0[r]], qb = q0[pc1[r]];
          const float qa1 = two_z ? q1[pc0[r]] : 0.f, qb1 = two_z ? q1[pc1[r]] : 0.f;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int v = 4 * r + i;
            float t = ra[v] * qa;
            t = fmaf(rb[v], qb, t);
            float val = u0 * t;
            if (two_z) {
              float bb = ra[v] * qa1;
              bb = fmaf(rb[v], qb1, bb);
              val = fmaf(u1, bb, val);
            }
            if (val != 0.f) acc[v] = fmaf(a[v], val, acc[v]);
          }
        }
        return;
      }
#pragma unroll
      for (int v = 0; v < kScVox; ++v) {
        float t = w0[v] * q0[l0[v]];
        t = fmaf(w1[v], q0[l1[v]], t);
        float val = u0 * t;
        if (two_z) {
          float bb = w0[v] * q1[l0[v]];
          bb = fmaf(w1[v], q1[l1[v]], bb);
          val = fmaf(u1, bb, val);
        }
        if (val != 0.f) acc[v] = fmaf(a[v], val, acc[v]);
      }
    };
    if (staged) {
      // shared-memory operands only (the pointers below are derived from the shared array)
      int s = 0;              // stage of group kk (kk mod n_stages, kept incrementally)
      uint32_t fph = 0;       // bit s: parity of the next phase of full[s]
      for (int g = g_begin; g < g_end; ++g, s = s + 1 == n_stages ? 0 : s + 1) {
        const int kk = g - g_begin;
        if (!bk_wait(full + s, (fph >> s) & 1u, abort_flag, polls)) {
          bad = true;
          break;
        }
        fph ^= 1u << s;
        unsigned char* st = stage(s);
        if (lf0 < l_end) {
          const TE* at = reinterpret_cast<const TE*>(st) + (lf0 - l_begin);
          float a[kScVox];
          load4x2(at, a);
          accumulate(a, reinterpret_cast<const float*>(st + seg_off) - cs0 + sh0,
                     reinterpret_cast<const float*>(st + seg_off + seg_bytes) - cs0 + sh1);
        }
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(empty + s);
          if (warp == 0) *used = kk + 1;
        }
      }
    } else if (lf0 < l_end) {
      for (int g = g_begin; g < g_end; ++g) {
        float a[kScVox];
        const TE* ag = eff + clamp_row(grow[g], n_det) * ld_eff + j0 + (lf0 - l_begin);
        if (run1) {
          load4x2(ag, a);
        } else {  // the second run would read past the tile (and possibly the row)
          float h[4];
          smem4(ag, 0, h);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            a[i] = h[i];
            a[4 + i] = 0.f;
          }
        }
        accumulate(a, q + (int64_t)g * ldq + (int64_t)z0 * n_lc, q + (int64_t)g * ldq + (int64_t)z1 * n_lc);
      }
    }
    if (bad) *abort_flag = 1;
    if (!bad) {
      float* out = part + (int64_t)blockIdx.y * ldp + (int64_t)zf * n_lf;
#pragma unroll
      for (int v = 0; v < kScVox; ++v)
        if (vox(v) < l_end) out[vox(v)] = acc[v];
    }
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    for (int kk = *used; kk < *issued; ++kk)
      mbar_wait_bounded(full + kk % n_stages, (kk / n_stages) & 1, kBkDrainPolls);
  }
}

// Scatter for the stride-4 ring stencil: the same CTA layout as the bulk scatter with
// sixteen voxels per thread (runs of four at stride 128, tiles of kSpTile fine voxels, q
// segments up to kSpSeg coarse values). Every run of four theta-consecutive voxels of a ring
// interpolates between two coarse voxels, so each voxel keeps two folded weights (ra, rb) and
// its sum in registers and a run reads two q values per z tap; the arithmetic per voxel is the
// bulk scatter's pair form (the same result). A thread whose runs are not pairs (tap tables
// that do not follow the stencil) reads its taps from global memory on every group instead.
constexpr int kSpVox = 16;
constexpr int kSpRuns = kSpVox / 4;
constexpr int kSpTile = kScConsumers * kSpVox;
constexpr int kSpSeg = 2048;

template <typename TE>
__global__ void __launch_bounds__(kScThreads, 2)
sparse_group_scatter_pair_kernel(const float* __restrict__ q, int64_t ldq, const int32_t* __restrict__ grow,
                                 int n_groups, int groups_per_chunk, const TE* __restrict__ eff, int64_t ld_eff,
                                 int64_t n_det, UpTaps taps, float* __restrict__ part, int64_t ldp,
                                 uint32_t stage_space, uint32_t seg_off) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);  // [kScMaxStages]
  uint64_t* empty = full + kScMaxStages;               // [kScMaxStages]
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 16 * kScMaxStages);
  int* issued = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 4);
  int* used = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 8);
  int* span = reinterpret_cast<int*>(smem + 16 * kScMaxStages + 12);  // [lmin, lmax]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t polls = g_bk_poll_limit;
  const int n_lf = taps.n_lf, n_lc = taps.n_lc;
  const int tiles_per_plane = (n_lf + kSpTile - 1) / kSpTile;
  const int zf = blockIdx.x / tiles_per_plane;
  const int l_begin = (blockIdx.x - zf * tiles_per_plane) * kSpTile;
  const int l_end = min(l_begin + kSpTile, n_lf);
  const int64_t j0 = (int64_t)zf * n_lf + l_begin;
  const int z0 = taps.zt[2 * zf], z1 = taps.zt[2 * zf + 1];
  const float u0 = taps.zwt[2 * zf], u1 = taps.zwt[2 * zf + 1];
  const bool two_z = u1 != 0.f;
  const int g_begin = blockIdx.y * groups_per_chunk;
  const int g_end = min(g_begin + groups_per_chunk, n_groups);
  if (tid == 0) {
    for (int s = 0; s < kScMaxStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, kScConsumers / 32);
    }
    *abort_flag = 0;
    *issued = *used = 0;
    span[0] = INT_MAX;
    span[1] = -1;
    mbar_init_fence();
  }
  __syncthreads();
  // this thread's voxels: runs r of four at lf0 + 128 r (one tap of the warp's voxels reads
  // consecutive q words; each run is one 8-byte sysmat load)
  const int lf0 = l_begin + warp * (32 * kSpVox) + lane * 4;
  auto vox = [&](int v) { return lf0 + (v >> 2) * 128 + (v & 3); };
  int pc0[kSpRuns], pc1[kSpRuns];
  float ra[kSpVox], rb[kSpVox];
  bool pair = true;
  if (tid < kScConsumers) {
    int mn = INT_MAX, mx = -1;
#pragma unroll
    for (int r = 0; r < kSpRuns; ++r) {
      int a = -1, b = -1;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int v = 4 * r + i, lf = vox(v);
        ra[v] = rb[v] = 0.f;
        if (lf >= l_end) continue;
        const int t[2] = {taps.lt[2 * lf], taps.lt[2 * lf + 1]};
        const float w[2] = {taps.lwt[2 * lf], taps.lwt[2 * lf + 1]};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          mn = min(mn, t[h]);
          mx = max(mx, t[h]);
          if (a < 0) a = t[h];
          if (t[h] == a) {
            ra[v] += w[h];
          } else {
            if (b < 0) b = t[h];
            if (t[h] == b) rb[v] += w[h];
            else pair = false;
          }
        }
      }
      pc0[r] = a < 0 ? 0 : a;
      pc1[r] = b < 0 ? pc0[r] : b;
    }
    if (mx >= 0) {
      atomicMin(span, mn);
      atomicMax(span + 1, mx);
    }
  }
  __syncthreads();
  const int cs0 = span[0] & ~3;
  const int seg_len = span[1] < 0 ? 4 : ((span[1] + 1 - cs0 + 3) & ~3);
  if (pair && tid < kScConsumers) {
#pragma unroll
    for (int r = 0; r < kSpRuns; ++r) {  // runs past the tile: indices inside the segment (weight 0)
      if (vox(4 * r) >= l_end) pc0[r] = pc1[r] = cs0;
    }
  }
  const bool staged = seg_len <= kSpSeg;
  const uint32_t a_bytes = (uint32_t)((l_end - l_begin) * sizeof(TE));
  const uint32_t seg_bytes = (uint32_t)seg_len * 4u;
  const uint32_t stage_bytes = (seg_off + seg_bytes * (two_z ? 2u : 1u) + 127u) & ~127u;
  int n_stages = (int)(stage_space / stage_bytes);
  if (n_stages > kScMaxStages) n_stages = kScMaxStages;
  if (n_stages < 1) n_stages = 1;  // (a tile that is not staged uses none)
  auto stage = [&](int s) { return smem + kScHeader + (size_t)s * stage_bytes; };
  if (warp == kScConsumers / 32) {
    // ------------------------------------------------------------ producer warp
    if (staged) {
      bool ok = true;
      int s = 0;
      uint32_t eph = 0;  // bit s: parity of the next phase of empty[s] to wait for
      for (int w = g_begin; w < g_end && ok; w += 32) {
        const int gv = w + lane < g_end ? grow[w + lane] : 0;  // 32 group rows per load
        const int m = min(32, g_end - w);
        for (int k = 0; k < m && ok; ++k) {
          const int row = __shfl_sync(0xffffffffu, gv, k);
          const int kk = w - g_begin + k;
          if (lane == 0) {
            if (kk >= n_stages) {
              ok = bk_wait(empty + s, (eph >> s) & 1u, abort_flag, polls);
              eph ^= 1u << s;
            }
            if (ok) {
              unsigned char* st = stage(s);
              const float* qg = q + (int64_t)(w + k) * ldq;
              mbar_arrive_expect_tx(full + s, a_bytes + seg_bytes * (two_z ? 2u : 1u));
              bulk_copy_g2s(st, eff + clamp_row(row, n_det) * ld_eff + j0, a_bytes, full + s);
              bulk_copy_g2s(st + seg_off, qg + (int64_t)z0 * n_lc + cs0, seg_bytes, full + s);
              if (two_z) bulk_copy_g2s(st + seg_off + seg_bytes, qg + (int64_t)z1 * n_lc + cs0, seg_bytes, full + s);
              *issued = kk + 1;
            }
          }
          s = s + 1 == n_stages ? 0 : s + 1;
          ok = __shfl_sync(0xffffffffu, ok, 0);
        }
      }
      if (!ok && lane == 0) *abort_flag = 1;
    }
  } else {
    // ------------------------------------------------------------ consumer warps
    float acc[kSpVox];
#pragma unroll
    for (int v = 0; v < kSpVox; ++v) acc[v] = 0.f;
    bool bad = false;
    // acc[v] += a[v] * (u0 * (ra qa + rb qb) + u1 * (ra qa1 + rb qb1)) per run (a: the run's
    // four sysmat values at ar), the scalar form of the bulk scatter's pair branch
    auto run = [&](int r, const float (&a)[4], const float* q0, const float* q1) {
      if (pair) {
        if (!two_z) {
          const float2 qa = make_float2(q0[pc0[r]], q0[pc0[r]]), qb = make_float2(q0[pc1[r]], q0[pc1[r]]);
#pragma unroll
          for (int i = 0; i < 4; i += 2) {
            const int v = 4 * r + i;
            float2 t = __fmul2_rn(make_float2(ra[v], ra[v + 1]), qa);
            t = __ffma2_rn(make_float2(rb[v], rb[v + 1]), qb, t);
            const float2 val = __fmul2_rn(make_float2(u0, u0), t);
            const float2 nw = __ffma2_rn(make_float2(a[i], a[i + 1]), val, make_float2(acc[v], acc[v + 1]));
            if (val.x != 0.f) acc[v] = nw.x;
            if (val.y != 0.f) acc[v + 1] = nw.y;
          }
        } else {
          const float qa = q0[pc0[r]], qb = q0[pc1[r]], qa1 = q1[pc0[r]], qb1 = q1[pc1[r]];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int v = 4 * r + i;
            float t = ra[v] * qa;
            t = fmaf(rb[v], qb, t);
            float val = u0 * t;
            float bb = ra[v] * qa1;
            bb = fmaf(rb[v], qb1, bb);
            val = fmaf(u1, bb, val);
            if (val != 0.f) acc[v] = fmaf(a[i], val, acc[v]);
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int v = 4 * r + i, lf = vox(v);
          if (lf >= l_end) continue;
          const int l0 = taps.lt[2 * lf], l1 = taps.lt[2 * lf + 1];
          const float w0 = taps.lwt[2 * lf], w1 = taps.lwt[2 * lf + 1];
          float t = w0 * q0[l0];
          t = fmaf(w1, q0[l1], t);
          float val = u0 * t;
          if (two_z) {
            float bb = w0 * q1[l0];
            bb = fmaf(w1, q1[l1], bb);
            val = fmaf(u1, bb, val);
          }
          if (val != 0.f) acc[v] = fmaf(a[i], val, acc[v]);
        }
      }
    };
    if (staged) {
      // shared-memory operands only (the pointers below are derived from the shared array)
      int s = 0;
      uint32_t fph = 0;  // bit s: parity of the next phase of full[s]
      for (int g = g_begin; g < g_end; ++g, s = s + 1 == n_stages ? 0 : s + 1) {
        const int kk = g - g_begin;
        if (!bk_wait(full + s, (fph >> s) & 1u, abort_flag, polls)) {
          bad = true;
          break;
        }
        fph ^= 1u << s;
        unsigned char* st = stage(s);
        const TE* at = reinterpret_cast<const TE*>(st) + (lf0 - l_begin);
        const float* q0 = reinterpret_cast<const float*>(st + seg_off) - cs0;
        const float* q1 = reinterpret_cast<const float*>(st + seg_off + seg_bytes) - cs0;
#pragma unroll
        for (int r = 0; r < kSpRuns; ++r)
          if (vox(4 * r) < l_end) {
            float a[4];
            smem4(at + 128 * r, 0, a);
            run(r, a, q0, q1);
          }
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(empty + s);
          if (warp == 0) *used = kk + 1;
        }
      }
    } else {
      for (int g = g_begin; g < g_end; ++g) {
        const TE* ag = eff + clamp_row(grow[g], n_det) * ld_eff + j0 + (lf0 - l_begin);
        const float* q0 = q + (int64_t)g * ldq + (int64_t)z0 * n_lc;
        const float* q1 = q + (int64_t)g * ldq + (int64_t)z1 * n_lc;
#pragma unroll
        for (int r = 0; r < kSpRuns; ++r)
          if (vox(4 * r) < l_end) {  // (runs are whole: the plane's length is a multiple of 4)
            float a[4];
            smem4(ag + 128 * r, 0, a);
            run(r, a, q0, q1);
          }
      }
    }
    if (bad) *abort_flag = 1;
    if (!bad) {
      float* out = part + (int64_t)blockIdx.y * ldp + (int64_t)zf * n_lf;
#pragma unroll
      for (int v = 0; v < kSpVox; ++v)
        if (vox(v) < l_end) out[vox(v)] = acc[v];
    }
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    for (int kk = *used; kk < *issued; ++kk)
      mbar_wait_bounded(full + kk % n_stages, (kk / n_stages) & 1, kBkDrainPolls);
  }
}

#include "sparse_cluster.cuh"

constexpr int kCfMaxClusters = 64;  // partial images reserved for the one-wave kernels (clusters, bulk scatters)
static bool g_cluster_fused = false;  // opt-in (jscc_set_fused_cluster)

// Co-resident clusters of the fused kernel for this device and shared-memory size (cached).
template <int MODE>
static int cf_max_clusters(size_t smem) {
  static int cache_dev[64] = {0};
  static size_t cache_smem[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (cache_dev[dev] > 0 && cache_smem[dev] == smem) return cache_dev[dev];
  if (cudaFuncSetAttribute(sparse_cluster_fused_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(num_sms() / kCfCluster * kCfCluster));
  cfg.blockDim = dim3(kCfThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCfCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, sparse_cluster_fused_kernel<MODE>, &cfg) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 0;
  }
  cache_dev[dev] = n;
  cache_smem[dev] = smem;
  return n;
}

static int64_t group_chunks(int64_t n_groups, int64_t vf) {
  const int64_t tiles = (vf + 255) / 256;
  int64_t chunks = (2432 + tiles - 1) / (tiles > 0 ? tiles : 1);  // ~16 CTAs x 152 SMs
  const int64_t max_chunks = (n_groups + 31) / 32;                 // >= 32 groups per chunk
  if (chunks > max_chunks) chunks = max_chunks;
  return chunks < 1 ? 1 : chunks;
}


template <typename TE, typename TC>
static int grouped_launch(const SpRows<TC>& rows, bool vec_rows, int64_t n_events, const int32_t* order,
                          const int32_t* goff, const int32_t* grow, int32_t n_groups, const TE* eff, int64_t ld_eff,
                          const UpTaps& taps, const int32_t* tj, const float* tw, int K, int ring_len,
                          int ring_stride, int64_t vf, int64_t vc, int32_t mode, const float* x, float* s_ev,
                          int have_sums, const int64_t* rotmat_inv,
                          int64_t ld_rot, float scale, float* weight, void* workspace, size_t workspace_bytes,
                          cudaStream_t st) {
  const int64_t ldp = (int64_t)align_up((size_t)vf, 8);
  const int64_t ldq = (int64_t)align_up((size_t)vc, 8);
  Carver cv(workspace, workspace_bytes);
  cv.take<float>((size_t)ldp);  // rotated image slot (used by the caller)
  float* coef = cv.take<float>((size_t)n_events);
  float* xw = cv.take<float>((size_t)K * vc);
  float* q = cv.take<float>((size_t)n_groups * ldq);
  const int64_t chunks = group_chunks(n_groups, vf);
  float* part = cv.take<float>((size_t)chunks * ldp);
  JSCC_REQUIRE(cv.ok(), "jscc_sparse_weight_grouped: workspace too small");
  const size_t smem = align_up((size_t)vc, 4) * sizeof(float);
  JSCC_REQUIRE(smem <= 227 * 1024, "jscc_sparse_weight_grouped: coarse grid (%zu bytes) exceeds shared memory", smem);
  int64_t per_sm = (227 * 1024) / (int64_t)(smem + 1024);
  if (per_sm > 8) per_sm = 8;
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)num_sms() * per_sm;
  if (grid > n_groups) grid = n_groups;
  // bulk-copy pipeline when every row start and length is 16-byte aligned (split storage),
  // b and q fit the event threads' registers and b plus at least two coarse rows fit in
  // shared memory
  // rows and b_g move in whole 16-byte units: a row's storage (its leading dimension) must
  // cover the rounded-up length; the kernel masks the values past vc
  const uint32_t row_bytes = (uint32_t)align_up((size_t)vc * sizeof(TC), 16);
  const uint32_t b_bytes = (uint32_t)align_up((size_t)vc * 4, 16);
  const uint32_t slot_off = (uint32_t)align_up(kBkHeader + align_up(b_bytes, 128), 128);
  const uint32_t slot_stride = (uint32_t)align_up(row_bytes, 128);
  const size_t bk_limit = 227 * 1024;
  int n_slots = 0;
  if (slot_off < bk_limit && slot_stride > 0) {
    n_slots = (int)((bk_limit - slot_off) / (size_t)slot_stride);
    if (n_slots > kBkMaxSlots) n_slots = kBkMaxSlots;
  }
  // events of a chunk: a power of two leaving as many slots in flight as it holds
  int batch = 1;
  while (batch * 2 <= kBkMaxBatch && batch * 2 <= n_slots / 2) batch *= 2;
  const bool bulk = rows.packed == nullptr && n_slots >= 2 && vc <= kBkMaxCoarse &&
                    reinterpret_cast<uintptr_t>(rows.tc) % 16 == 0 && (rows.ld * sizeof(TC)) % 16 == 0 &&
                    (size_t)rows.ld * sizeof(TC) >= row_bytes && reinterpret_cast<uintptr_t>(eff) % 16 == 0 &&
                    (ld_eff * sizeof(TE)) % 16 == 0 && ((size_t)vf * sizeof(TE)) % 16 == 0 && ldq % 4 == 0;
  const size_t bk_smem = (size_t)slot_off + (size_t)n_slots * slot_stride;
  int64_t bk_grid = num_sms();
  if (bk_grid > n_groups) bk_grid = n_groups;
  const int M = (K + 1) / 2;
  int4* tpx = cv.take<int4>((size_t)M * vc);  // packed taps with x folded in
  int4* tpw = cv.take<int4>((size_t)M * vc);  // packed taps, weights only (row sums)
  float4* xsx = cv.take<float4>((size_t)2 * vc);  // ring stencil, x folded in
  float4* xsw = cv.take<float4>((size_t)2 * vc);  // ring stencil, weights only
  // partial images of the one-wave kernels (the cluster path or the bulk scatters), one per
  // cluster or chunk of groups
  float* part_cf = cv.take<float>((size_t)kCfMaxClusters * ldp);
  float* bq = cv.take<float>((size_t)n_groups * ldq);             // group adjoints b_g (bulk path)
  JSCC_REQUIRE(cv.ok(), "jscc_sparse_weight_grouped: workspace too small");
  // stride-4 ring stencil (checked by the caller against the tap table): centres multiples of 4
  bool ring = bulk && ring_stride == 4 && K == 7 && ring_len >= 8 && ring_len % 4 == 0 &&
              taps.n_lf % ring_len == 0 && taps.n_lc * 4 == taps.n_lf && vf / taps.n_lf == vc / taps.n_lc &&
              vf < (1 << 30);
  // adjoint tiles of whole rings (at most kAdVox * kAdCompute coarse voxels, an even number so
  // that every segment starts on a 16-byte boundary), chunks of groups for about three CTAs per SM
  int ad_tile = 0, ad_tiles = 0, ad_chunks = 1, ad_gpc = 0, ad_stages = 0;
  uint32_t ad_stride = 0;
  size_t ad_smem = 0;
  if (ring) {
    const int n_thc = ring_len / 4;
    const int n_blocks = (int)(vc / n_thc);
    const int rmax = (kAdVox * kAdCompute) / n_thc;
    if (rmax >= 1) {
      ad_tiles = (n_blocks + rmax - 1) / rmax;
      int r = (n_blocks + ad_tiles - 1) / ad_tiles;
      if ((r * n_thc) % 2 != 0) ++r;
      if (r * n_thc > kAdVox * kAdCompute) r -= 2;
      ad_tile = r * n_thc;
    }
    ring = ad_tile > 0 && ad_tile % 2 == 0;
    if (ring) {
      ad_tiles = (int)((vc + ad_tile - 1) / ad_tile);
      ad_stride = (uint32_t)align_up((size_t)ad_tile * 4 * sizeof(TE), 128);
      ad_stages = (int)((74u * 1024u - kAdHeader) / ad_stride);  // three CTAs per SM
      if (ad_stages > kAdMaxStages) ad_stages = kAdMaxStages;
      if (ad_stages < 2) ad_stages = 2;
      ad_smem = kAdHeader + (size_t)ad_stages * ad_stride;
      ring = ad_smem <= 227 * 1024;
      int64_t ch = (3 * (int64_t)num_sms()) / ad_tiles;  // one wave of about three CTAs per SM
      if (ch > n_groups) ch = n_groups;
      ad_chunks = (int)(ch < 1 ? 1 : ch);
      ad_gpc = (int)((n_groups + ad_chunks - 1) / ad_chunks);
    }
  }
  {
    int64_t blocks = ((int64_t)K * vc + 255) / 256;
    if (blocks > (int64_t)num_sms() * 8) blocks = (int64_t)num_sms() * 8;
    if (ring) {
      JSCC_TIMED("sparse_fold_x", st,
                 (sparse_fold_ring_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, K, (int)vc, taps.n_lc, taps.n_lf,
                                                                            ring_len, x, xsx)));
      JSCC_LAUNCH_CHECK();
      if (mode == JSCC_SPARSE_MATERIALIZE && !have_sums) {
        JSCC_TIMED("sparse_fold_x", st,
                   (sparse_fold_ring_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, K, (int)vc, taps.n_lc,
                                                                              taps.n_lf, ring_len, nullptr, xsw)));
        JSCC_LAUNCH_CHECK();
      }
    } else if (bulk) {
      JSCC_TIMED("sparse_fold_x", st,
                 (sparse_fold_pack_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, K, M, vc, x, tpx)));
      JSCC_LAUNCH_CHECK();
      if (mode == JSCC_SPARSE_MATERIALIZE && !have_sums) {
        JSCC_TIMED("sparse_fold_x", st,
                   (sparse_fold_pack_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, K, M, vc, nullptr, tpw)));
        JSCC_LAUNCH_CHECK();
      }
    } else {
      JSCC_TIMED("sparse_fold_x", st,
                 (sparse_fold_x_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, (int64_t)K * vc, x, xw)));
      JSCC_LAUNCH_CHECK();
    }
  }
  cudaError_t attr = cudaSuccess;
#define JSCC_GA(TP, XS)                                                                                          \
  do {                                                                                                           \
    if (ring) {                                                                                                  \
      attr = cudaFuncSetAttribute(sparse_group_adjoint_ring_kernel<TE>,                                          \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ad_smem);                    \
      if (attr == cudaSuccess)                                                                                   \
        JSCC_TIMED("sparse_group_adjoint", st,                                                                   \
                   (sparse_group_adjoint_ring_kernel<TE><<<dim3((unsigned)ad_tiles, (unsigned)ad_chunks),        \
                                                           kAdThreads, ad_smem, st>>>(                           \
                       grow, n_groups, ad_gpc, eff, ld_eff, rows.n_det, XS, (int)vc, ad_tile, ring_len, bq, ldq, \
                       ad_stages, ad_stride)));                                                                  \
    } else {                                                                                                     \
      const dim3 ag((unsigned)((vc + 255) / 256), (unsigned)(n_groups < 65535 ? n_groups : 65535));            \
      if (K <= 4)                                                                                                \
        JSCC_TIMED("sparse_group_adjoint", st,                                                                   \
                   (sparse_group_adjoint_taps_kernel<4, TE><<<ag, 256, 0, st>>>(grow, n_groups, eff, ld_eff,     \
                                                                             rows.n_det, TP, M, (int)vc, bq,    \
                                                                             ldq)));                            \
      else if (K <= 8)                                                                                           \
        JSCC_TIMED("sparse_group_adjoint", st,                                                                   \
                   (sparse_group_adjoint_taps_kernel<8, TE><<<ag, 256, 0, st>>>(grow, n_groups, eff, ld_eff,     \
                                                                             rows.n_det, TP, M, (int)vc, bq,    \
                                                                             ldq)));                            \
      else                                                                                                       \
        JSCC_TIMED("sparse_group_adjoint", st,                                                                   \
                   (sparse_group_adjoint_taps_kernel<0, TE><<<ag, 256, 0, st>>>(grow, n_groups, eff, ld_eff,     \
                                                                             rows.n_det, TP, M, (int)vc, bq,    \
                                                                             ldq)));                            \
    }                                                                                                            \
  } while (0)
#define JSCC_GC_BK(MODE, TP, XS)                                                                                 \
  do {                                                                                                           \
    JSCC_GA(TP, XS);                                                                                             \
    if (attr == cudaSuccess) attr = cudaGetLastError();                                                          \
    if (vc % 4 == 0) {                                                                                           \
      if (attr == cudaSuccess)                                                                                   \
        attr = cudaFuncSetAttribute(sparse_group_coef_bulk_kernel<MODE, TC, false>,                              \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bk_smem);                  \
      if (attr == cudaSuccess)                                                                                   \
        JSCC_TIMED(MODE == 2 ? "sparse_group_rowsum" : "sparse_group_coef", st,                                  \
                   (sparse_group_coef_bulk_kernel<MODE, TC, false><<<(unsigned)bk_grid, kBkThreads, bk_smem,     \
                                                                     st>>>(                                     \
                       rows, order, goff, n_groups, (int)vc, bq, s_ev, q, ldq, n_slots, batch, b_bytes,         \
                       row_bytes, slot_off, slot_stride)));                                                     \
    } else {                                                                                                     \
      if (attr == cudaSuccess)                                                                                   \
        attr = cudaFuncSetAttribute(sparse_group_coef_bulk_kernel<MODE, TC, true>,                               \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bk_smem);                  \
      if (attr == cudaSuccess)                                                                                   \
        JSCC_TIMED(MODE == 2 ? "sparse_group_rowsum" : "sparse_group_coef", st,                                  \
                   (sparse_group_coef_bulk_kernel<MODE, TC, true><<<(unsigned)bk_grid, kBkThreads, bk_smem,      \
                                                                    st>>>(                                      \
                       rows, order, goff, n_groups, (int)vc, bq, s_ev, q, ldq, n_slots, batch, b_bytes,         \
                       row_bytes, slot_off, slot_stride)));                                                     \
    }                                                                                                            \
  } while (0)
#define JSCC_GC_K(MODE, KT, TW)                                                                                  \
  do {                                                                                                           \
    attr = cudaFuncSetAttribute(sparse_group_coef_kernel<MODE, KT, TE, TC>,                                      \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                         \
    if (attr == cudaSuccess)                                                                                     \
      JSCC_TIMED(MODE == 2 ? "sparse_group_rowsum" : "sparse_group_coef", st,                                    \
                 (sparse_group_coef_kernel<MODE, KT, TE, TC><<<(unsigned)grid, kGcThreads, smem, st>>>(          \
                     rows, vec_rows, order, goff, grow, n_groups, vc, tj, TW, K, eff, ld_eff, s_ev, coef, q,     \
                     ldq)));                                                                                     \
  } while (0)
#define JSCC_GC(MODE, TW, TP, XS)                                                                                \
  do {                                                                                                           \
    if (bulk) {                                                                                                  \
      JSCC_GC_BK(MODE, TP, XS);                                                                                  \
    } else if (K <= 4) JSCC_GC_K(MODE, 4, TW);                                                                   \
    else if (K <= 8) JSCC_GC_K(MODE, 8, TW);                                                                     \
    else JSCC_GC_K(MODE, 0, TW);                                                                                 \
  } while (0)
  // ---- fused cluster path (one kernel: coefficients and scatter; see sparse_cluster.cuh):
  // BF16 split rows and sysmat, one plane of rings under the stride-4 ring stencil, slices
  // and windows that fit the kernel's registers and shared memory
  if constexpr (std::is_same<TE, __nv_bfloat16>::value && std::is_same<TC, __nv_bfloat16>::value) {
    const int n_rings = ring ? (int)(vf / ring_len) : 0;
    bool cf_ok = g_cluster_fused && ring && taps.n_lf == vf && vf % 8 == 0 && vc % 8 == 0 && n_rings >= kCfCluster &&
                 vf < (1 << 24);
    int max_wf = 0, max_wc = 0;
    if (cf_ok) {
      for (int r = 0; r < kCfCluster; ++r) {
        const CfSlice s = cf_slice(r, n_rings, ring_len, (int)vf, (int)vc);
        max_wf = std::max(max_wf, s.jw1 - s.jw0);
        max_wc = std::max(max_wc, s.cw1 - s.cw0);
        cf_ok = cf_ok && (s.J1 - s.J0) <= kCfMaxSliceF;
      }
      cf_ok = cf_ok && max_wc <= kCfMaxWindowC;
    }
    CfArgs ca{};
    size_t cf_smem = 0;
    if (cf_ok) {
      ca.x_off = kCfHeader;
      ca.erow_off = ca.x_off + (uint32_t)align_up((size_t)max_wf * 4, 128);
      ca.erow_stride = (uint32_t)align_up((size_t)max_wf * 2, 128);
      ca.b_off = ca.erow_off + 3 * ca.erow_stride;
      ca.b_stride = (uint32_t)align_up((size_t)max_wc * 4, 128);
      ca.q_off = ca.b_off + 2 * ca.b_stride;
      ca.q_stride = ca.b_stride;
      ca.slot_off = ca.q_off + 4 * ca.q_stride;  // q: [group parity][event team]
      ca.slot_stride = (uint32_t)align_up((size_t)max_wc * 2, 128);
      const size_t limit = 227 * 1024;
      int ns = ca.slot_off < limit ? (int)((limit - ca.slot_off) / ca.slot_stride) : 0;
      ns = std::min(ns, kCfMaxSlots);
      ca.n_slots = ns;
      cf_smem = (size_t)ca.slot_off + (size_t)ns * ca.slot_stride;
      cf_ok = ns >= 2 * kCfNB;
    }
    int n_clusters = 0;
    if (cf_ok) {
      n_clusters = mode == JSCC_SPARSE_MATERIALIZE ? cf_max_clusters<0>(cf_smem) : cf_max_clusters<1>(cf_smem);
      n_clusters = std::min(std::min(n_clusters, kCfMaxClusters), (int)n_groups);
      cf_ok = n_clusters >= 1;
    }
    if (cf_ok) {
      if (mode == JSCC_SPARSE_MATERIALIZE && !have_sums) {
        JSCC_GC(2, tw, tpw, xsw);  // S_i = t_i . adj(A_g), kept by the caller across calls
        JSCC_CUDA_CHECK(attr);
        JSCC_LAUNCH_CHECK();
      }
      ca.tc = rows.tc;
      ca.ld = rows.ld;
      ca.n_det = rows.n_det;
      ca.order = order;
      ca.goff = goff;
      ca.grow = grow;
      ca.n_groups = n_groups;
      ca.eff = eff;
      ca.ld_eff = ld_eff;
      ca.x = x;
      ca.s_ev = s_ev;
      ca.part = part_cf;
      ca.ldp = ldp;
      ca.vf = (int)vf;
      ca.vc = (int)vc;
      ca.ring_len = ring_len;
      ca.n_rings = n_rings;
      ca.max_wf = max_wf;
      ca.max_wc = max_wc;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)(n_clusters * kCfCluster));
      cfg.blockDim = dim3(kCfThreads);
      cfg.dynamicSmemBytes = cf_smem;
      cfg.stream = st;
      cudaLaunchAttribute cattr[1];
      cattr[0].id = cudaLaunchAttributeClusterDimension;
      cattr[0].val.clusterDim.x = kCfCluster;
      cattr[0].val.clusterDim.y = 1;
      cattr[0].val.clusterDim.z = 1;
      cfg.attrs = cattr;
      cfg.numAttrs = 1;
      if (mode == JSCC_SPARSE_MATERIALIZE)
        JSCC_TIMED("sparse_group_fused", st, (attr = cudaLaunchKernelEx(&cfg, sparse_cluster_fused_kernel<0>, ca)));
      else
        JSCC_TIMED("sparse_group_fused", st, (attr = cudaLaunchKernelEx(&cfg, sparse_cluster_fused_kernel<1>, ca)));
      JSCC_CUDA_CHECK(attr);
      JSCC_LAUNCH_CHECK();
      int64_t blocks = (vf + 255) / 256;
      if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
      const int has_scale = scale != 1.0f;
      JSCC_TIMED("sparse_reduce", st,
                 (sparse_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part_cf, ldp, n_clusters, rotmat_inv, ld_rot,
                                                                         vf, has_scale, scale, weight)));
      JSCC_LAUNCH_CHECK();
      return JSCC_OK;
    }
  }
  if (mode == JSCC_SPARSE_MATERIALIZE) {
    if (!have_sums) {
      JSCC_GC(2, tw, tpw, xsw);  // S_i = t_i . adj(A_g), kept by the caller across calls
      JSCC_CUDA_CHECK(attr);
      JSCC_LAUNCH_CHECK();
    }
    JSCC_GC(0, xw, tpx, xsx);
  } else {
    JSCC_GC(1, xw, tpx, xsx);
  }
#undef JSCC_GC
#undef JSCC_GC_K
#undef JSCC_GC_BK
#undef JSCC_GA
  JSCC_CUDA_CHECK(attr);
  JSCC_LAUNCH_CHECK();
  const int gpc = (int)((n_groups + chunks - 1) / chunks);
  // bulk scatter when the sysmat tiles and the q segments start on 16-byte boundaries
  // (one q segment per stage when the coarse grid has one z plane, else two; stages to
  // ~98 KB so that two CTAs share an SM)
  const int n_zc = (int)(vc / taps.n_lc);
  const uint32_t sc_a = (uint32_t)align_up((size_t)kScTile * sizeof(TE), 128);
  const uint32_t sc_stage = sc_a + (n_zc > 1 ? 2u : 1u) * kScSeg * 4u;  // largest stage
  // two CTAs per SM: the kernel packs its stages into the space (at least two of the largest)
  const size_t sc_smem = 110u * 1024u;
  const uint32_t sc_space = (uint32_t)(sc_smem - kScHeader);
  const bool sc_bulk = sc_space >= 2 * sc_stage && reinterpret_cast<uintptr_t>(eff) % 16 == 0 && (ld_eff * sizeof(TE)) % 16 == 0 &&
                       ((size_t)taps.n_lf * sizeof(TE)) % 16 == 0 && taps.n_lf % kScVox == 0 &&
                       taps.n_lf >= kScTile / 2 &&  // tiles never span z planes: short planes idle them
                       reinterpret_cast<uintptr_t>(q) % 16 == 0 && ldq % 4 == 0;
  int64_t n_part = chunks;
  float* part_out = part;
  // the stride-4 ring stencil's scatter: sixteen voxels per thread (the kernel checks that every
  // run of four interpolates between two coarse voxels and reads the taps itself otherwise)
  const uint32_t sp_a = (uint32_t)align_up((size_t)kSpTile * sizeof(TE), 128);
  const bool sc_pair = sc_bulk && taps.n_lc % 4 == 0 && ring_stride == 4 && ring_len >= 8 && ring_len % 4 == 0 &&
                       taps.n_lf % ring_len == 0 && taps.n_lc * 4 == taps.n_lf &&
                       sc_space >= 2 * (sp_a + (n_zc > 1 ? 2u : 1u) * kSpSeg * 4u);
  if (sc_pair) {
    const int tiles = (int)(vf / taps.n_lf) * ((taps.n_lf + kSpTile - 1) / kSpTile);
    // one wave: tiles x chunks <= two CTAs per SM, partial images in the one-wave slots
    int64_t sc_chunks = 2 * (int64_t)num_sms() / tiles;
    if (sc_chunks > kCfMaxClusters) sc_chunks = kCfMaxClusters;
    if (sc_chunks > n_groups) sc_chunks = n_groups;
    if (sc_chunks < 1) sc_chunks = 1;
    const int sc_gpc = (int)((n_groups + sc_chunks - 1) / sc_chunks);
    JSCC_CUDA_CHECK(cudaFuncSetAttribute(sparse_group_scatter_pair_kernel<TE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem));
    JSCC_TIMED("sparse_group_scatter", st,
               (sparse_group_scatter_pair_kernel<TE><<<dim3((unsigned)tiles, (unsigned)sc_chunks), kScThreads,
                                                       sc_smem, st>>>(q, ldq, grow, n_groups, sc_gpc, eff, ld_eff,
                                                                      rows.n_det, taps, part_cf, ldp, sc_space, sp_a)));
    n_part = sc_chunks;
    part_out = part_cf;
  } else if (sc_bulk) {
    const int tiles = (int)(vf / taps.n_lf) * ((taps.n_lf + kScTile - 1) / kScTile);
    // one wave: tiles x chunks <= two CTAs per SM, partial images in the one-wave slots
    int64_t sc_chunks = 2 * (int64_t)num_sms() / tiles;
    if (sc_chunks > kCfMaxClusters) sc_chunks = kCfMaxClusters;
    if (sc_chunks > n_groups) sc_chunks = n_groups;
    if (sc_chunks < 1) sc_chunks = 1;
    const int sc_gpc = (int)((n_groups + sc_chunks - 1) / sc_chunks);
    JSCC_CUDA_CHECK(cudaFuncSetAttribute(sparse_group_scatter_bulk_kernel<TE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem));
    JSCC_TIMED("sparse_group_scatter", st,
               (sparse_group_scatter_bulk_kernel<TE><<<dim3((unsigned)tiles, (unsigned)sc_chunks), kScThreads,
                                                       sc_smem, st>>>(q, ldq, grow, n_groups, sc_gpc, eff, ld_eff,
                                                                      rows.n_det, taps, part_cf, ldp, sc_space, sc_a)));
    n_part = sc_chunks;
    part_out = part_cf;
  } else {
    dim3 sgrid((unsigned)((vf + 255) / 256), (unsigned)chunks);
    JSCC_TIMED("sparse_group_scatter", st,
               (sparse_group_scatter_kernel<TE><<<sgrid, 256, 0, st>>>(q, ldq, grow, n_groups, gpc, vf, eff, ld_eff,
                                                                       rows.n_det, taps, part, ldp)));
  }
  JSCC_LAUNCH_CHECK();
  int64_t blocks = (vf + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  const int has_scale = scale != 1.0f;
  JSCC_TIMED("sparse_reduce", st,
             (sparse_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part_out, ldp, (int)n_part, rotmat_inv, ld_rot, vf,
                                                                     has_scale, scale, weight)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

}  // namespace jscc

using namespace jscc;

extern "C" {

int jscc_sparse_map(const void* in, int32_t in_dtype, int64_t ld_in, const int32_t* row_idx, int64_t n_rows,
                    float* out, int64_t ld_out, const int32_t* z_ptr, const int32_t* z_idx, const float* z_w,
                    int32_t n_zo, int32_t n_zi, const int32_t* l_ptr, const int32_t* l_idx, const float* l_w,
                    int32_t n_lo, int32_t n_li, void* stream) {
  JSCC_REQUIRE(n_rows >= 0 && n_zo >= 0 && n_lo >= 0 && n_zi >= 0 && n_li >= 0, "jscc_sparse_map: negative size");
  JSCC_REQUIRE(in_dtype == JSCC_DTYPE_F32 || in_dtype == JSCC_DTYPE_BF16, "jscc_sparse_map: bad dtype");
  if (n_rows == 0 || (int64_t)n_zo * n_lo == 0) return JSCC_OK;
  JSCC_REQUIRE(in && out && z_ptr && z_idx && z_w && l_ptr && l_idx && l_w, "jscc_sparse_map: null pointer argument");
  JSCC_REQUIRE(ld_in >= (int64_t)n_zi * n_li && ld_out >= (int64_t)n_zo * n_lo, "jscc_sparse_map: bad leading dims");
  JSCC_REQUIRE(n_rows <= 65535, "jscc_sparse_map: at most 65,535 rows per call");
  cudaStream_t st = as_stream(stream);
  const int64_t n_out = (int64_t)n_zo * n_lo;
  int64_t bx = (n_out + 255) / 256;
  if (bx > 128) bx = 128;
  dim3 grid((unsigned)bx, (unsigned)n_rows);
  if (in_dtype == JSCC_DTYPE_F32)
    JSCC_TIMED("sparse_map", st,
               (sparse_map_kernel<float><<<grid, 256, 0, st>>>(static_cast<const float*>(in), ld_in, row_idx, n_rows,
                                                               out, ld_out, z_ptr, z_idx, z_w, n_zo, l_ptr, l_idx, l_w,
                                                               n_lo, n_li)));
  else
    JSCC_TIMED("sparse_map", st,
               (sparse_map_kernel<__nv_bfloat16><<<grid, 256, 0, st>>>(
                   static_cast<const __nv_bfloat16*>(in), ld_in, row_idx, n_rows, out, ld_out, z_ptr, z_idx, z_w, n_zo,
                   l_ptr, l_idx, l_w, n_lo, n_li)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_sparse_pack(const int64_t* cp1, const float* t_compton, int64_t ld_tc, int64_t n_events, int64_t n_coarse,
                     float* rows, int64_t ld_rows, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_coarse >= 0, "jscc_sparse_pack: negative size");
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(cp1 && rows && (t_compton || n_coarse == 0), "jscc_sparse_pack: null pointer argument");
  JSCC_REQUIRE(ld_rows >= n_coarse + 1 && ld_tc >= n_coarse, "jscc_sparse_pack: bad leading dims");
  JSCC_REQUIRE(n_events <= 65535, "jscc_sparse_pack: at most 65,535 events per call");
  cudaStream_t st = as_stream(stream);
  int64_t bx = (n_coarse + 1 + 255) / 256;
  if (bx > 64) bx = 64;
  dim3 grid((unsigned)bx, (unsigned)n_events);
  JSCC_TIMED("sparse_pack", st,
             (sparse_pack_kernel<<<grid, 256, 0, st>>>(cp1, t_compton, ld_tc, n_events, n_coarse, rows, ld_rows)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_sparse_unpack_ids(const float* rows, int64_t ld_rows, int64_t n_events, int64_t* cp1, void* stream) {
  JSCC_REQUIRE(n_events >= 0, "jscc_sparse_unpack_ids: negative size");
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(rows && cp1, "jscc_sparse_unpack_ids: null pointer argument");
  cudaStream_t st = as_stream(stream);
  int64_t b = (n_events + 255) / 256;
  if (b > 4096) b = 4096;
  JSCC_TIMED("sparse_unpack", st, (sparse_unpack_kernel<<<(unsigned)b, 256, 0, st>>>(rows, ld_rows, n_events, cp1)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

static int make_taps(const int32_t* z_taps, const float* z_tw, const int32_t* l_taps, const float* l_tw,
                     int32_t n_lf, int32_t n_lc, UpTaps* t) {
  JSCC_REQUIRE(z_taps && z_tw && l_taps && l_tw, "sparse upsample taps missing");
  JSCC_REQUIRE(n_lf > 0 && n_lc > 0, "sparse upsample layer sizes must be positive");
  t->zt = z_taps;
  t->zwt = z_tw;
  t->lt = l_taps;
  t->lwt = l_tw;
  t->n_lf = n_lf;
  t->n_lc = n_lc;
  return JSCC_OK;
}

int jscc_sparse_materialize(const float* rows, int64_t ld_rows, int64_t n_events, const void* sysmat,
                            int32_t sysmat_dtype, int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps,
                            const float* z_tw, int32_t n_zf, const int32_t* l_taps, const float* l_tw, int32_t n_lf,
                            int32_t n_lc, float* fine, int64_t ld_fine, float* row_sum, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det > 0, "jscc_sparse_materialize: bad sizes");
  JSCC_REQUIRE(sysmat_dtype == JSCC_DTYPE_F32 || sysmat_dtype == JSCC_DTYPE_BF16, "jscc_sparse_materialize: dtype");
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(rows && sysmat && fine && row_sum, "jscc_sparse_materialize: null pointer argument");
  UpTaps t;
  const int rc = make_taps(z_taps, z_tw, l_taps, l_tw, n_lf, n_lc, &t);
  if (rc != JSCC_OK) return rc;
  const int64_t vf = (int64_t)n_zf * n_lf;
  JSCC_REQUIRE(ld_fine >= vf && ld_sysmat >= vf, "jscc_sparse_materialize: bad leading dims");
  JSCC_REQUIRE(n_events <= 2147483647LL, "jscc_sparse_materialize: too many events");
  cudaStream_t st = as_stream(stream);
  if (sysmat_dtype == JSCC_DTYPE_F32)
    JSCC_TIMED("sparse_materialize", st,
               (sparse_materialize_kernel<float><<<(unsigned)n_events, 256, 0, st>>>(
                   rows, ld_rows, n_events, vf, static_cast<const float*>(sysmat), ld_sysmat, n_det, t, fine, ld_fine,
                   row_sum)));
  else
    JSCC_TIMED("sparse_materialize", st,
               (sparse_materialize_kernel<__nv_bfloat16><<<(unsigned)n_events, 256, 0, st>>>(
                   rows, ld_rows, n_events, vf, static_cast<const __nv_bfloat16*>(sysmat), ld_sysmat, n_det, t, fine,
                   ld_fine, row_sum)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

size_t jscc_sparse_weight_workspace_bytes(int64_t n_events, int64_t n_fine) {
  return plan_sparse(n_events, n_fine).ws_bytes;
}

int jscc_sparse_weight(const float* rows, int64_t ld_rows, int64_t n_events, const void* sysmat, int32_t sysmat_dtype,
                       int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps, const float* z_tw, int32_t n_zf,
                       const int32_t* l_taps, const float* l_tw, int32_t n_lf, int32_t n_lc, int32_t mode,
                       const float* img, const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, float scale,
                       float* weight, void* workspace, size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det > 0, "jscc_sparse_weight: bad sizes");
  JSCC_REQUIRE(mode == JSCC_SPARSE_MATERIALIZE || mode == JSCC_SPARSE_GROUPED, "jscc_sparse_weight: bad mode %d",
               mode);
  JSCC_REQUIRE(sysmat_dtype == JSCC_DTYPE_F32 || sysmat_dtype == JSCC_DTYPE_BF16, "jscc_sparse_weight: dtype");
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(rows && sysmat && img && weight, "jscc_sparse_weight: null pointer argument");
  JSCC_REQUIRE((rotmat == nullptr) == (rotmat_inv == nullptr), "jscc_sparse_weight: give both rotation tables");
  UpTaps t;
  int rc = make_taps(z_taps, z_tw, l_taps, l_tw, n_lf, n_lc, &t);
  if (rc != JSCC_OK) return rc;
  const int64_t vf = (int64_t)n_zf * n_lf;
  JSCC_REQUIRE(ld_sysmat >= vf, "jscc_sparse_weight: ld_sysmat < fine voxels");
  SpRows<float> r{rows, nullptr, nullptr, ld_rows, n_det};
  return sparse_weight_impl<float>(r, n_events, sysmat, sysmat_dtype, ld_sysmat, t, vf, mode, img, rotmat, rotmat_inv,
                                   ld_rot, scale, weight, workspace, workspace_bytes, as_stream(stream));
}

int jscc_sparse_weight_split(const int32_t* row_id, const void* t_coarse, int32_t tc_dtype, int64_t ld_tc,
                             int64_t n_events, const void* sysmat, int32_t sysmat_dtype, int64_t ld_sysmat,
                             int64_t n_det, const int32_t* z_taps, const float* z_tw, int32_t n_zf,
                             const int32_t* l_taps, const float* l_tw, int32_t n_lf, int32_t n_lc, int32_t mode,
                             const float* img, const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot,
                             float scale, float* weight, void* workspace, size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det > 0, "jscc_sparse_weight_split: bad sizes");
  JSCC_REQUIRE(mode == JSCC_SPARSE_MATERIALIZE || mode == JSCC_SPARSE_GROUPED, "jscc_sparse_weight_split: mode");
  JSCC_REQUIRE(sysmat_dtype == JSCC_DTYPE_F32 || sysmat_dtype == JSCC_DTYPE_BF16, "jscc_sparse_weight_split: dtype");
  JSCC_REQUIRE(tc_dtype == JSCC_DTYPE_F32 || tc_dtype == JSCC_DTYPE_BF16, "jscc_sparse_weight_split: row dtype");
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(row_id && t_coarse && sysmat && img && weight, "jscc_sparse_weight_split: null pointer argument");
  JSCC_REQUIRE((rotmat == nullptr) == (rotmat_inv == nullptr), "jscc_sparse_weight_split: give both tables");
  UpTaps t;
  int rc = make_taps(z_taps, z_tw, l_taps, l_tw, n_lf, n_lc, &t);
  if (rc != JSCC_OK) return rc;
  const int64_t vf = (int64_t)n_zf * n_lf;
  JSCC_REQUIRE(ld_sysmat >= vf, "jscc_sparse_weight_split: ld_sysmat < fine voxels");
  JSCC_REQUIRE(ld_tc >= (int64_t)n_lc * (n_zf > 0 ? 1 : 0), "jscc_sparse_weight_split: ld_tc too small");
  if (tc_dtype == JSCC_DTYPE_F32) {
    SpRows<float> r{nullptr, row_id, static_cast<const float*>(t_coarse), ld_tc, n_det};
    return sparse_weight_impl<float>(r, n_events, sysmat, sysmat_dtype, ld_sysmat, t, vf, mode, img, rotmat,
                                     rotmat_inv, ld_rot, scale, weight, workspace, workspace_bytes, as_stream(stream));
  }
  SpRows<__nv_bfloat16> r{nullptr, row_id, static_cast<const __nv_bfloat16*>(t_coarse), ld_tc, n_det};
  return sparse_weight_impl<__nv_bfloat16>(r, n_events, sysmat, sysmat_dtype, ld_sysmat, t, vf, mode, img, rotmat,
                                           rotmat_inv, ld_rot, scale, weight, workspace, workspace_bytes,
                                           as_stream(stream));
}


size_t jscc_sparse_grouped_workspace_bytes(int64_t n_events, int64_t n_fine, int64_t n_coarse, int32_t n_groups,
                                           int32_t adj_width) {
  const int64_t ldp = (int64_t)align_up((size_t)(n_fine > 0 ? n_fine : 1), 8);
  const int64_t ldq = (int64_t)align_up((size_t)(n_coarse > 0 ? n_coarse : 1), 8);
  const int64_t chunks = group_chunks(n_groups, n_fine);
  return align_up((size_t)ldp * sizeof(float), 256) + align_up((size_t)(n_events > 0 ? n_events : 1) * 4, 256) +
         align_up((size_t)(adj_width > 0 ? adj_width : 1) * (n_coarse > 0 ? n_coarse : 1) * 4, 256) +
         align_up((size_t)(n_groups > 0 ? n_groups : 1) * ldq * sizeof(float), 256) +
         align_up((size_t)chunks * ldp * sizeof(float), 256) +
         2 * align_up((size_t)((adj_width > 0 ? adj_width : 1) + 1) / 2 * (n_coarse > 0 ? n_coarse : 1) * 16, 256) +
         2 * align_up((size_t)(n_coarse > 0 ? n_coarse : 1) * 32, 256) +
         align_up((size_t)kCfMaxClusters * ldp * sizeof(float), 256) +
         align_up((size_t)(n_groups > 0 ? n_groups : 1) * ldq * sizeof(float), 256) + 256;
}

int jscc_set_fused_cluster(int32_t enable) {
  jscc::g_cluster_fused = enable != 0;
  return JSCC_OK;
}

int jscc_sparse_weight_grouped(const int32_t* row_id, const void* t_coarse, int32_t tc_dtype, int64_t ld_tc,
                               const float* packed_rows, int64_t n_events, const int32_t* order,
                               const int32_t* group_offsets, const int32_t* group_rows, int32_t n_groups,
                               float* event_sums, int32_t have_sums, const void* sysmat, int32_t sysmat_dtype,
                               int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps, const float* z_tw, int32_t n_zf,
                               const int32_t* l_taps, const float* l_tw, int32_t n_lf, int32_t n_lc, int32_t n_zc,
                               const int32_t* adj_idx, const float* adj_w, int32_t adj_width, int32_t ring_len,
                               int32_t ring_stride, int32_t mode, const float* img, const int64_t* rotmat,
                               const int64_t* rotmat_inv, int64_t ld_rot, float scale, float* weight, void* workspace,
                               size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det > 0 && n_groups >= 0, "jscc_sparse_weight_grouped: bad sizes");
  JSCC_REQUIRE(ring_len >= 0 && ring_stride >= 0, "jscc_sparse_weight_grouped: negative ring description");
  JSCC_REQUIRE(mode == JSCC_SPARSE_MATERIALIZE || mode == JSCC_SPARSE_GROUPED, "jscc_sparse_weight_grouped: mode");
  JSCC_REQUIRE(sysmat_dtype == JSCC_DTYPE_F32 || sysmat_dtype == JSCC_DTYPE_BF16, "jscc_sparse_weight_grouped: dtype");
  if (n_events == 0 || n_groups == 0) return JSCC_OK;
  JSCC_REQUIRE(order && group_offsets && group_rows && sysmat && img && weight,
               "jscc_sparse_weight_grouped: null pointer argument");
  JSCC_REQUIRE(mode == JSCC_SPARSE_GROUPED || event_sums, "jscc_sparse_weight_grouped: event_sums needed");
  JSCC_REQUIRE(packed_rows || (row_id && t_coarse), "jscc_sparse_weight_grouped: rows missing");
  JSCC_REQUIRE(packed_rows || tc_dtype == JSCC_DTYPE_F32 || tc_dtype == JSCC_DTYPE_BF16,
               "jscc_sparse_weight_grouped: row dtype");
  JSCC_REQUIRE(adj_idx && adj_w && adj_width > 0 && adj_width <= 64,
               "jscc_sparse_weight_grouped: adjoint tap table missing or wider than 64");
  JSCC_REQUIRE((rotmat == nullptr) == (rotmat_inv == nullptr), "jscc_sparse_weight_grouped: give both tables");
  UpTaps t;
  int rc = make_taps(z_taps, z_tw, l_taps, l_tw, n_lf, n_lc, &t);
  if (rc != JSCC_OK) return rc;
  const int64_t vf = (int64_t)n_zf * n_lf;
  const int64_t vc = (int64_t)n_zc * n_lc;
  JSCC_REQUIRE(ld_sysmat >= vf, "jscc_sparse_weight_grouped: ld_sysmat < fine voxels");
  const size_t need = jscc_sparse_grouped_workspace_bytes(n_events, vf, vc, n_groups, adj_width);
  JSCC_REQUIRE(workspace && workspace_bytes >= need, "jscc_sparse_weight_grouped: workspace too small (%zu < %zu)",
               workspace_bytes, need);
  cudaStream_t st = as_stream(stream);
  const int64_t ldp = (int64_t)align_up((size_t)vf, 8);
  Carver cv0(workspace, workspace_bytes);
  float* xr = cv0.take<float>((size_t)ldp);  // same first slot as grouped_launch's carve
  const float* x = img;
  if (rotmat) {
    int64_t blocks = (vf + 255) / 256;
    if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
    JSCC_TIMED("sc_gather_rot", st,
               (sc_gather_rot_kernel<<<(unsigned)blocks, 256, 0, st>>>(img, rotmat, ld_rot, 0, 1, vf, ldp, xr)));
    JSCC_LAUNCH_CHECK();
    x = xr;
  }
  const size_t tcsz = packed_rows ? 4 : (tc_dtype == JSCC_DTYPE_BF16 ? 2 : 4);
  const bool vec_rows = !packed_rows && (ld_tc * (int64_t)tcsz) % 16 == 0 &&
                        reinterpret_cast<uintptr_t>(t_coarse) % 16 == 0;
#define JSCC_GROUPED(TE, TC, ROWS)                                                                             \
  grouped_launch<TE, TC>(ROWS, vec_rows, n_events, order, group_offsets, group_rows, n_groups,                 \
                         static_cast<const TE*>(sysmat), ld_sysmat, t, adj_idx, adj_w, adj_width, ring_len,      \
                         ring_stride, vf, vc, mode,                                                              \
                         x, event_sums, have_sums, rotmat_inv, ld_rot, scale, weight, workspace,                 \
                         workspace_bytes, st)
  if (packed_rows) {
    SpRows<float> r{packed_rows, nullptr, nullptr, ld_tc, n_det};
    return sysmat_dtype == JSCC_DTYPE_F32 ? JSCC_GROUPED(float, float, r) : JSCC_GROUPED(__nv_bfloat16, float, r);
  }
  if (tc_dtype == JSCC_DTYPE_F32) {
    SpRows<float> r{nullptr, row_id, static_cast<const float*>(t_coarse), ld_tc, n_det};
    return sysmat_dtype == JSCC_DTYPE_F32 ? JSCC_GROUPED(float, float, r) : JSCC_GROUPED(__nv_bfloat16, float, r);
  }
  SpRows<__nv_bfloat16> r{nullptr, row_id, static_cast<const __nv_bfloat16*>(t_coarse), ld_tc, n_det};
  return sysmat_dtype == JSCC_DTYPE_F32 ? JSCC_GROUPED(float, __nv_bfloat16, r)
                                        : JSCC_GROUPED(__nv_bfloat16, __nv_bfloat16, r);
#undef JSCC_GROUPED
}

}  // extern "C"

namespace jscc {
// Poll bound of the bulk kernels' pipeline waits on the current device (`reset` restores
// the default).
int set_bulk_poll_limit(uint32_t polls, bool reset) {
  const uint32_t v = reset ? kBkMaxPolls : polls;
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_bk_poll_limit, &v, sizeof(v)));
  return JSCC_OK;
}
int take_sc_timeout_count(unsigned int* out);  // sc_projector.cu
}  // namespace jscc

extern "C" {

int jscc_take_wait_timeout_count(unsigned int* out) {
  JSCC_REQUIRE(out, "jscc_take_wait_timeout_count: null pointer argument");
  unsigned int h = 0, zero = 0, hs = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_wait_timeout_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_wait_timeout_count, &zero, sizeof(zero)));
  const int rc = jscc::take_sc_timeout_count(&hs);  // the fused SC kernel's give-ups
  if (rc != JSCC_OK) return rc;
  *out = h + hs;
  return JSCC_OK;
}

}  // extern "C"
