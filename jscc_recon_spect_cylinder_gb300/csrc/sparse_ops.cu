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
#include "jscc_common.cuh"

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
          s_ev[i] = f;
        } else if (MODE == 0) {
          const float si = s_ev[i];
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
// The same per-group computation with every operand staged in shared memory by bulk copies
// (cp.async.bulk completing on mbarriers), so each byte is read from HBM once and the adjoint
// gather, the event dots and the q accumulation all read shared memory. One persistent CTA
// per SM walks its groups gi = blockIdx.x, + gridDim.x, ...; shared memory holds
//   erow  [vf] TE       the group's sysmat row; the next group's row is fetched as soon as
//                       the adjoint of the current one is done
//   b     [vc] float    adj(A_g * x) (MODE 2: adj(A_g))
//   slots [2][batch][vc] TC   coarse rows of two batches of (up to `batch`) events of one
//                       group: while one batch is used the next one, possibly of a later
//                       group, is in flight
// Dots: each thread owns four coarse values per 2048 and accumulates all the batch's events,
// partial sums are reduced per warp and then over warps in warp order (deterministic). q is
// accumulated over the group's events in event order, batch after batch, in the q row.
// Every wait is bounded: on a timeout the CTA counts it (jscc_take_wait_timeout_count),
// waits (bounded) for its copies still in flight and returns.
constexpr int kBkThreads = 512;
constexpr int kBkWarps = kBkThreads / 32;
constexpr int kBkMaxBatch = 8;
constexpr int kBkHeader = 1024;               // barriers, dot partials, coefficients, abort flag
constexpr uint32_t kBkMaxPolls = 1u << 22;    // per wait

__device__ unsigned int g_wait_timeout_count = 0;

// Adjoint of one group from the shared-memory sysmat row (plain loads; see group_adjoint).
template <int KT, typename TE>
__device__ __forceinline__ void group_adjoint_smem(float* b, int64_t vc, const int32_t* __restrict__ tj,
                                                   const float* __restrict__ tw, int K, const TE* er, int tid) {
  for (int64_t c0 = tid; c0 < vc; c0 += 2 * kBkThreads) {
    float acc[2] = {0.f, 0.f};
    if (KT > 0) {
      int idx[2][KT > 0 ? KT : 1];
      float wv[2][KT > 0 ? KT : 1];
#pragma unroll
      for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int64_t c = c0 + (int64_t)u * kBkThreads;
          const bool in = c < vc && k < K;  // the table has K rows; KT may exceed K
          idx[u][k] = in ? __ldg(tj + (int64_t)k * vc + c) : 0;
          wv[u][k] = in ? __ldg(tw + (int64_t)k * vc + c) : 0.f;
        }
#pragma unroll
      for (int k = 0; k < KT; ++k)
#pragma unroll
        for (int u = 0; u < 2; ++u) acc[u] = fmaf(wv[u][k], to_float(er[idx[u][k]]), acc[u]);
    } else {
      for (int k = 0; k < K; ++k)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int64_t c = c0 + (int64_t)u * kBkThreads;
          if (c < vc) {
            const float wvv = __ldg(tw + (int64_t)k * vc + c);
            if (wvv != 0.f) acc[u] = fmaf(wvv, to_float(er[__ldg(tj + (int64_t)k * vc + c)]), acc[u]);
          }
        }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t c = c0 + (int64_t)u * kBkThreads;
      if (c < vc) b[c] = acc[u];
    }
  }
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

template <int MODE, int KT, typename TE, typename TC>
__global__ void __launch_bounds__(kBkThreads, 1)
sparse_group_coef_bulk_kernel(SpRows<TC> rows, const int32_t* __restrict__ order, const int32_t* __restrict__ goff,
                              const int32_t* __restrict__ grow, int n_groups, int64_t vc,
                              const int32_t* __restrict__ tj, const float* __restrict__ tw, int K,
                              const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ s_ev,
                              float* __restrict__ q, int64_t ldq, int batch, uint32_t erow_bytes, uint32_t row_bytes,
                              uint32_t b_off, uint32_t slot_off, uint32_t slot_stride) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);  // [2][kBkMaxBatch] row slots, then the sysmat row
  uint64_t* ebar = bar + 2 * kBkMaxBatch;
  float* red = reinterpret_cast<float*>(smem + 256);  // [kBkWarps][kBkMaxBatch]
  float* cs = red + kBkWarps * kBkMaxBatch;           // [kBkMaxBatch]
  int* abort_flag = reinterpret_cast<int*>(cs + kBkMaxBatch);
  TE* erow = reinterpret_cast<TE*>(smem + kBkHeader);
  float* b = reinterpret_cast<float*>(smem + b_off);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = gridDim.x;
  auto slot = [&](int h, int k) { return reinterpret_cast<TC*>(smem + slot_off + (size_t)(h * batch + k) * slot_stride); };
  if (tid == 0) {
    for (int s = 0; s < 2 * kBkMaxBatch + 1; ++s) mbar_init(bar + s, 1);
    *abort_flag = 0;
    mbar_init_fence();
  }
  __syncthreads();
  // ---- producer state (thread 0): the last batch issued and the barriers with a copy in flight
  uint32_t pending = 0;
  int ig = blockIdx.x, ib = ig < n_groups ? goff[ig] : 0;
  auto seek = [&]() -> bool {  // (ig, ib) -> the first batch at or after it, skipping empty groups
    while (ig < n_groups) {
      if (ib < goff[ig + 1]) return true;
      ig += G;
      if (ig < n_groups) ib = goff[ig];
    }
    return false;
  };
  auto issue_row = [&](int gi) {
    mbar_arrive_expect_tx(ebar, erow_bytes);
    bulk_copy_g2s(erow, eff + clamp_row(grow[gi], rows.n_det) * ld_eff, erow_bytes, ebar);
    pending |= 1u << (2 * kBkMaxBatch);
  };
  auto issue_batch = [&](int h) {
    const int n = min(batch, goff[ig + 1] - ib);
    for (int k = 0; k < n; ++k) {
      uint64_t* bk = bar + h * kBkMaxBatch + k;
      mbar_arrive_expect_tx(bk, row_bytes);
      bulk_copy_g2s(slot(h, k), rows.coarse(order[ib + k]), row_bytes, bk);
      pending |= 1u << (h * kBkMaxBatch + k);
    }
  };
  if (tid == 0 && blockIdx.x < n_groups) {
    issue_row(blockIdx.x);
    if (seek()) issue_batch(0);
  }
  uint32_t ph = 0;  // parity of every barrier's next phase (bit s: barrier s)
  auto wait = [&](int s) {
    if (!mbar_wait_bounded(bar + s, (ph >> s) & 1u, kBkMaxPolls)) *abort_flag = 1;
    ph ^= 1u << s;
    pending &= ~(1u << s);
  };
  int nb = 0;  // batches consumed (selects the half)
  bool aborted = false;
  for (int gi = blockIdx.x; gi < n_groups && !aborted; gi += G) {
    wait(2 * kBkMaxBatch);
    group_adjoint_smem<KT, TE>(b, vc, tj, tw, K, erow, tid);
    __syncthreads();
    if (*abort_flag) { aborted = true; break; }
    if (tid == 0 && gi + G < n_groups) {
      fence_proxy_async_smem();
      issue_row(gi + G);
    }
    const int e0 = goff[gi], e1 = goff[gi + 1];
    float* qg = q + (int64_t)gi * ldq;
    if (MODE != 2 && e0 == e1)
      for (int64_t c = (int64_t)tid * 4; c < vc; c += kBkThreads * 4)
        *reinterpret_cast<float4*>(qg + c) = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int bs = e0; bs < e1; bs += batch, ++nb) {
      const int n = min(batch, e1 - bs), h = nb & 1;
      if (tid == 0) {  // the next batch into the other half (its last batch ended at the last barrier)
        ib += batch;
        if (seek()) {
          fence_proxy_async_smem();
          issue_batch(h ^ 1);
        }
      }
      for (int k = 0; k < n; ++k) wait(h * kBkMaxBatch + k);
      // ---- dots f_i = t_i . b
      float acc[kBkMaxBatch];
#pragma unroll
      for (int k = 0; k < kBkMaxBatch; ++k) acc[k] = 0.f;
      for (int64_t c = (int64_t)tid * 4; c < vc; c += kBkThreads * 4) {
        const float4 bv = *reinterpret_cast<const float4*>(b + c);
#pragma unroll
        for (int k = 0; k < kBkMaxBatch; ++k)
          if (k < n) {
            float v[4];
            smem4(slot(h, k), c, v);
            acc[k] = fmaf(v[0], bv.x, acc[k]);
            acc[k] = fmaf(v[1], bv.y, acc[k]);
            acc[k] = fmaf(v[2], bv.z, acc[k]);
            acc[k] = fmaf(v[3], bv.w, acc[k]);
          }
      }
#pragma unroll
      for (int k = 0; k < kBkMaxBatch; ++k)
        if (k < n) {
          const float f = warp_sum(acc[k]);
          if (lane == 0) red[warp * kBkMaxBatch + k] = f;
        }
      __syncthreads();
      if (*abort_flag) { aborted = true; break; }
      if (tid < n) {
        float f = 0.f;
        for (int w = 0; w < kBkWarps; ++w) f += red[w * kBkMaxBatch + tid];
        const int64_t i = order[bs + tid];
        if (MODE == 2) {
          s_ev[i] = f;
        } else if (MODE == 0) {
          const float si = s_ev[i];
          cs[tid] = (isfinite(si) && si > 0.f) ? (1.0f / fmaxf(f / si, 1e-12f)) / si : 0.f;
        } else {
          cs[tid] = 1.0f / fmaxf(f, 1e-12f);
        }
      }
      if (MODE != 2) {
        __syncthreads();
        // ---- q_g += sum over the batch of c_i t_i, events in order
        for (int64_t c = (int64_t)tid * 4; c < vc; c += kBkThreads * 4) {
          float4 a = bs == e0 ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(qg + c);
#pragma unroll
          for (int k = 0; k < kBkMaxBatch; ++k)
            if (k < n) {
              const float ck = cs[k];
              if (ck != 0.f) {
                float v[4];
                smem4(slot(h, k), c, v);
                a.x = fmaf(ck, v[0], a.x);
                a.y = fmaf(ck, v[1], a.y);
                a.z = fmaf(ck, v[2], a.z);
                a.w = fmaf(ck, v[3], a.w);
              }
            }
          *reinterpret_cast<float4*>(qg + c) = a;
        }
      }
      __syncthreads();  // the batch's slots and coefficients are free
    }
  }
  if (aborted && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    for (int s = 0; s <= 2 * kBkMaxBatch; ++s)  // copies still in flight write this CTA's memory
      if (pending & (1u << s)) mbar_wait_bounded(bar + s, (ph >> s) & 1u, kBkMaxPolls);
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
  float acc = 0.f;
#pragma unroll 4
  for (int gi = g_begin; gi < g_end; ++gi) {
    const float* qg = q + (int64_t)gi * ldq;
    float a = w0 * __ldg(qg + c00);
    a = fmaf(w1, __ldg(qg + c01), a);
    float v = u0 * a;
    if (u1 != 0.f) {
      float bb = w0 * __ldg(qg + c10);
      bb = fmaf(w1, __ldg(qg + c11), bb);
      v = fmaf(u1, bb, v);
    }
    if (v != 0.f) acc = fmaf(ld_any(eff + clamp_row(grow[gi], n_det) * ld_eff, j), v, acc);
  }
  part[(int64_t)blockIdx.y * ldp + j] = acc;
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
                          const UpTaps& taps, const int32_t* tj, const float* tw, int K, int64_t vf, int64_t vc,
                          int32_t mode, const float* x, float* s_ev, int have_sums, const int64_t* rotmat_inv,
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
  {
    const int64_t n = (int64_t)K * vc;
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)num_sms() * 8) blocks = (int64_t)num_sms() * 8;
    JSCC_TIMED("sparse_fold_x", st, (sparse_fold_x_kernel<<<(unsigned)blocks, 256, 0, st>>>(tj, tw, n, x, xw)));
    JSCC_LAUNCH_CHECK();
  }
  cudaError_t attr = cudaSuccess;
  // bulk-copy pipeline when every row start and length is 16-byte aligned (split storage)
  // and a sysmat row, b and two batches of coarse rows fit in shared memory
  const uint32_t erow_bytes = (uint32_t)((size_t)vf * sizeof(TE)), row_bytes = (uint32_t)((size_t)vc * sizeof(TC));
  const uint32_t b_off = (uint32_t)align_up(kBkHeader + align_up(erow_bytes, 128), 128);
  const uint32_t slot_off = (uint32_t)(b_off + align_up((size_t)vc * 4, 128));
  const uint32_t slot_stride = (uint32_t)align_up(row_bytes, 128);
  const size_t bk_limit = 227 * 1024;
  int batch = 0;
  if (slot_off < bk_limit && slot_stride > 0) {
    batch = (int)((bk_limit - slot_off) / (2 * (size_t)slot_stride));
    if (batch > kBkMaxBatch) batch = kBkMaxBatch;
  }
  const bool bulk = rows.packed == nullptr && batch >= 1 && (size_t)vf * sizeof(TE) < (1u << 20) &&
                    reinterpret_cast<uintptr_t>(rows.tc) % 16 == 0 && (rows.ld * sizeof(TC)) % 16 == 0 &&
                    row_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(eff) % 16 == 0 &&
                    (ld_eff * sizeof(TE)) % 16 == 0 && erow_bytes % 16 == 0;
  const size_t bk_smem = (size_t)slot_off + 2 * (size_t)batch * slot_stride;
  int64_t bk_grid = num_sms();
  if (bk_grid > n_groups) bk_grid = n_groups;
#define JSCC_GC_BK(MODE, KT, TW)                                                                                 \
  do {                                                                                                           \
    attr = cudaFuncSetAttribute(sparse_group_coef_bulk_kernel<MODE, KT, TE, TC>,                                 \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bk_smem);                      \
    if (attr == cudaSuccess)                                                                                     \
      JSCC_TIMED(MODE == 2 ? "sparse_group_rowsum" : "sparse_group_coef", st,                                    \
                 (sparse_group_coef_bulk_kernel<MODE, KT, TE, TC><<<(unsigned)bk_grid, kBkThreads, bk_smem,      \
                                                                     st>>>(                                      \
                     rows, order, goff, grow, n_groups, vc, tj, TW, K, eff, ld_eff, s_ev, q, ldq, batch,         \
                     erow_bytes, row_bytes, b_off, slot_off, slot_stride)));                                     \
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
#define JSCC_GC(MODE, TW)                                                                                        \
  do {                                                                                                           \
    if (bulk) {                                                                                                  \
      if (K <= 4) JSCC_GC_BK(MODE, 4, TW);                                                                       \
      else if (K <= 8) JSCC_GC_BK(MODE, 8, TW);                                                                  \
      else JSCC_GC_BK(MODE, 0, TW);                                                                              \
    } else if (K <= 4) JSCC_GC_K(MODE, 4, TW);                                                                   \
    else if (K <= 8) JSCC_GC_K(MODE, 8, TW);                                                                     \
    else JSCC_GC_K(MODE, 0, TW);                                                                                 \
  } while (0)
  if (mode == JSCC_SPARSE_MATERIALIZE) {
    if (!have_sums) {
      JSCC_GC(2, tw);  // S_i = t_i . adj(A_g), kept by the caller across calls
      JSCC_CUDA_CHECK(attr);
      JSCC_LAUNCH_CHECK();
    }
    JSCC_GC(0, xw);
  } else {
    JSCC_GC(1, xw);
  }
#undef JSCC_GC
#undef JSCC_GC_K
#undef JSCC_GC_BK
  JSCC_CUDA_CHECK(attr);
  JSCC_LAUNCH_CHECK();
  const int gpc = (int)((n_groups + chunks - 1) / chunks);
  dim3 sgrid((unsigned)((vf + 255) / 256), (unsigned)chunks);
  JSCC_TIMED("sparse_group_scatter", st,
             (sparse_group_scatter_kernel<TE><<<sgrid, 256, 0, st>>>(q, ldq, grow, n_groups, gpc, vf, eff, ld_eff,
                                                                     rows.n_det, taps, part, ldp)));
  JSCC_LAUNCH_CHECK();
  int64_t blocks = (vf + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  const int has_scale = scale != 1.0f;
  JSCC_TIMED("sparse_reduce", st,
             (sparse_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part, ldp, (int)chunks, rotmat_inv, ld_rot, vf,
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
         align_up((size_t)chunks * ldp * sizeof(float), 256) + 256;
}

int jscc_sparse_weight_grouped(const int32_t* row_id, const void* t_coarse, int32_t tc_dtype, int64_t ld_tc,
                               const float* packed_rows, int64_t n_events, const int32_t* order,
                               const int32_t* group_offsets, const int32_t* group_rows, int32_t n_groups,
                               float* event_sums, int32_t have_sums, const void* sysmat, int32_t sysmat_dtype,
                               int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps, const float* z_tw, int32_t n_zf,
                               const int32_t* l_taps, const float* l_tw, int32_t n_lf, int32_t n_lc, int32_t n_zc,
                               const int32_t* adj_idx, const float* adj_w, int32_t adj_width, int32_t mode,
                               const float* img, const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot,
                               float scale, float* weight, void* workspace, size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det > 0 && n_groups >= 0, "jscc_sparse_weight_grouped: bad sizes");
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
                         static_cast<const TE*>(sysmat), ld_sysmat, t, adj_idx, adj_w, adj_width, vf, vc, mode,  \
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

int jscc_take_wait_timeout_count(unsigned int* out) {
  JSCC_REQUIRE(out, "jscc_take_wait_timeout_count: null pointer argument");
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_wait_timeout_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_wait_timeout_count, &zero, sizeof(zero)));
  *out = h;
  return JSCC_OK;
}

}  // extern "C"
