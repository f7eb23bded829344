// Compton cone kernel (kernel a): per-event preparation, materialised T rows for the
// builders, and the fused list-mode weight w = T^T (1 / (T x)) with T recomputed on the fly.
//
// Reference semantics
//   strict:  process_list_plane_strict.py:151-253 (filters :164-189, theta :24-27, sigma_E
//            :39-52, sigma_pos :59-134, kernel :228), t = cone * sysmat[cp1 - 1] (:240)
//   legacy:  process_list_plane.py:17-107 (derivative sigma_E :66-74, atan sigma_pos :77-80)
//   simple:  exp(-(beta - theta)^2 / (2 sigma_E^2)) / d01^2 (the simplified kernel of the
//            list-mode benchmark description; strict records, no sigma_pos, no Klein-Nishina)
//   weight:  recon_osem_plane.py:33-42 (get_weight_compton) over the builder's rows; rows are
//            normalised there, and the list-mode weight is invariant to a row's scale, so the
//            fused form skips the normalisation.
//
// GB300 design
//   * One 64-byte record per event (positions, Compton angle, sigma branches, Klein-Nishina
//     factor, per-axis position variance, cos(beta) window). The Compton angle and its
//     energy-sigma branches are computed in FP64 on request (the 1/(E0 - E1) difference
//     loses bits in FP32 near the Compton edge); event-selection decisions are made in
//     FP32 with the reference's operation order so the surviving event set is identical.
//   * Window: sigma_pos is bounded per event by sqrt(max_k s_k) / d12 (|grad beta| = 1/d12)
//     and sigma_E by max(sigma+, sigma-), so |beta - theta| > K sigma_max implies
//     t < exp(-K^2/2). Pairs whose cos(beta) falls outside the window skip acos/exp and
//     the efficiency load (K = window_sigmas; K <= 0 evaluates every pair).
//   * Forward: CTA = 256 threads x EB events; every thread walks voxels, keeps EB partial
//     sums in registers, fixed-order CTA reduction at the end.
//   * Back: CTA = 256 voxels x one event chunk; partial column sums per chunk to the
//     workspace, then the chunk-ordered reduce of sc_projector.cu (shared kernel).
//   No float atomics; results are bit-reproducible.
#include "jscc_common.cuh"

namespace jscc {

// Shared with sc_projector.cu.
__global__ void sc_gather_rot_kernel(const float* __restrict__ img, const int64_t* __restrict__ rotmat,
                                     int64_t ld_rot, int r0, int nr, int64_t V, int64_t ldx,
                                     float* __restrict__ xr);
__global__ void sc_reduce_scatter_kernel(const float* __restrict__ part, int64_t ldp, int chunks,
                                         int nr, int rb_stride, const int64_t* __restrict__ rotinv,
                                         int64_t ld_rot, int r0, int64_t V, int has_scale,
                                         float scale, float* __restrict__ weight);

__device__ unsigned int g_bad_detector_count = 0;

struct alignas(16) ConeEvent {
  float p1x, p1y, p1z;     // first-hit position
  float vx, vy, vz;        // v12 = pos2 - pos1
  float d12;               // |v12|
  float theta;             // Compton angle
  float sig_plus, sig_minus;
  float kn;                // e0 / (e0 - e1) + (e0 - e1) / e0
  float s0, s1, s2;        // strict: sigma1^2 + sigma2^2 per axis; legacy: delta_r1, q, cos(theta)
  float cos_lo, cos_hi;    // cos(beta) window
};
static_assert(sizeof(ConeEvent) == 64, "record layout");

constexpr float kEE = 0.511f;

// ------------------------------------------------------------------ event preparation
__device__ __forceinline__ float compton_cos_f32(float e1, float e0) {
  // 1 - ((ee * e1) / ((e0 - e1) * e0)), each operation rounded as the reference's tensor ops
  return __fsub_rn(1.0f, __fdiv_rn(__fmul_rn(kEE, e1), __fmul_rn(__fsub_rn(e0, e1), e0)));
}

__device__ __forceinline__ double compton_theta_f64(double e1, double e0) {
  double c = 1.0 - (0.511 * e1) / ((e0 - e1) * e0);
  c = fmin(fmax(c, -1.0 + 1e-7), 1.0 - 1e-7);
  return acos(c);
}

__device__ __forceinline__ float compton_theta_f32(float e1, float e0) {
  float c = compton_cos_f32(e1, e0);
  c = fminf(fmaxf(c, -1.0f + 1e-7f), 1.0f - 1e-7f);
  return acosf(c);
}

__global__ void compton_event_prep_kernel(const float* __restrict__ list, int64_t ld_list, int64_t n,
                                          const float* __restrict__ det, const float* __restrict__ sig1,
                                          const float* __restrict__ sig2, int64_t n_det, float e0, float res,
                                          float thr_max, float thr_min, float thr_sum, int model, int theta_fp64,
                                          float window_k, float dr1, float dr2, uint8_t* __restrict__ keep,
                                          ConeEvent* __restrict__ rec, int32_t* __restrict__ row_id) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float* L = list + i * ld_list;
    const int cp1 = (int)L[0];  // torch .int(): truncation toward zero
    const int cp2 = (int)L[2];
    const float e1 = L[1], e2 = L[3];
    bool k = (e1 < thr_max) && (e1 > thr_min) && (e2 > thr_min) && (__fadd_rn(e1, e2) > thr_sum);
    if (model != 1) {
      const float c = compton_cos_f32(e1, e0);
      k = k && (c > -1.0f + 1e-6f) && (c < 1.0f - 1e-6f);
    }
    if (cp1 < 1 || cp1 > n_det || cp2 < 1 || cp2 > n_det) {
      if (k) atomicAdd(&g_bad_detector_count, 1u);
      k = false;
    }
    if (k) {
      const float y1 = det[(int64_t)(cp1 - 1) * 3 + 1], y2 = det[(int64_t)(cp2 - 1) * 3 + 1];
      k = fabsf(__fsub_rn(y1, y2)) > 0.1f;
    }
    keep[i] = k ? 1 : 0;
    row_id[i] = k ? cp1 - 1 : 0;
    if (!k) continue;
    ConeEvent r;
    const float* a = det + (int64_t)(cp1 - 1) * 3;
    const float* b = det + (int64_t)(cp2 - 1) * 3;
    r.p1x = a[0]; r.p1y = a[1]; r.p1z = a[2];
    r.vx = __fsub_rn(b[0], a[0]);
    r.vy = __fsub_rn(b[1], a[1]);
    r.vz = __fsub_rn(b[2], a[2]);
    r.d12 = sqrtf(r.vx * r.vx + r.vy * r.vy + r.vz * r.vz);
    if (model != 1) {
      // sigma_E: e1 -/+ e1 * res / 2.355 * sqrt(e0 / e1), clamped to (1e-7, e0 - 1e-7)
      if (theta_fp64) {
        const double E0 = (double)e0, E1 = (double)e1;
        const double th = compton_theta_f64(E1, E0);
        const double se = E1 * (double)res / 2.355 * sqrt(E0 / E1);
        const double lo = fmin(fmax(E1 - se, 1e-7), E0 - 1e-7);
        const double hi = fmin(fmax(E1 + se, 1e-7), E0 - 1e-7);
        r.theta = (float)th;
        r.sig_minus = (float)fmax(th - compton_theta_f64(lo, E0), 1e-7);
        r.sig_plus = (float)fmax(compton_theta_f64(hi, E0) - th, 1e-7);
        r.kn = (float)(E0 / (E0 - E1) + (E0 - E1) / E0);
      } else {
        const float th = compton_theta_f32(e1, e0);
        const float se = e1 * res / 2.355f * sqrtf(e0 / e1);
        const float lo = fminf(fmaxf(e1 - se, 1e-7f), e0 - 1e-7f);
        const float hi = fminf(fmaxf(e1 + se, 1e-7f), e0 - 1e-7f);
        r.theta = th;
        r.sig_minus = fmaxf(th - compton_theta_f32(lo, e0), 1e-7f);
        r.sig_plus = fmaxf(compton_theta_f32(hi, e0) - th, 1e-7f);
        r.kn = e0 / (e0 - e1) + (e0 - e1) / e0;
      }
      const float* q1 = sig1 + (int64_t)(cp1 - 1) * 3;
      const float* q2 = sig2 + (int64_t)(cp2 - 1) * 3;
      r.s0 = q1[0] + q2[0];
      r.s1 = q1[1] + q2[1];
      r.s2 = q1[2] + q2[2];
      if (window_k > 0.f) {
        const float d12c = fmaxf(r.d12, 1e-7f);
        const float smax = fmaxf(fmaxf(r.s0, r.s1), r.s2);
        const float sp2 = smax / (d12c * d12c);
        const float se = fmaxf(r.sig_plus, r.sig_minus);
        // 1 % margin on the bound for rounding in the per-pair terms
        const float sig_max = 1.01f * sqrtf(fmaxf(sp2 + se * se, 1e-12f));
        const float hi_ang = fminf(r.theta + window_k * sig_max, 3.14159265f);
        const float lo_ang = fmaxf(r.theta - window_k * sig_max, 0.f);
        r.cos_lo = hi_ang >= 3.14159265f ? -2.f : cosf(hi_ang);
        r.cos_hi = lo_ang <= 0.f ? 2.f : cosf(lo_ang);
      } else {
        r.cos_lo = -2.f;
        r.cos_hi = 2.f;
      }
    } else {
      // legacy: unclamped theta and first/second-derivative sigma_E (process_list_plane.py:64-74)
      const float th = acosf(compton_cos_f32(e1, e0));
      const float er = e1 * res / 2.355f * sqrtf(e0 / e1);
      const float st = sinf(th), ct = cosf(th);
      const float dm = e0 - e1;
      const float dth = (1.0f / fabsf(st)) * kEE / (dm * dm);
      const float d2th = kEE / (st * dm * dm * dm) * (2.0f - ct / (st * st) * kEE / dm);
      r.theta = th;
      r.sig_plus = fabsf(dth * er + 0.5f * d2th * er * er);
      r.sig_minus = fabsf(dth * er - 0.5f * d2th * er * er);
      r.kn = e0 / dm + dm / e0;
      r.s0 = dr1;
      r.s1 = dr1 / dr2;
      r.s2 = ct;
      r.cos_lo = -2.f;
      r.cos_hi = 2.f;
    }
    rec[i] = r;
  }
}

// ------------------------------------------------------------------ per-pair kernel value
// Returns the cone value t_ij (no efficiency factor). WINDOW: skip outside the cos window.
template <int MODEL, bool WINDOW>
__device__ __forceinline__ float cone_value(const ConeEvent& e, float cx, float cy, float cz) {
  const float ax = e.p1x - cx, ay = e.p1y - cy, az = e.p1z - cz;
  const float dot = ax * e.vx + ay * e.vy + az * e.vz;
  const float d01sq = ax * ax + ay * ay + az * az;
  const float d01 = sqrtf(d01sq);
  if (MODEL == 0) {
    const float bcos = dot / fmaxf(d01 * e.d12, 1e-7f);
    if (WINDOW && (bcos < e.cos_lo || bcos > e.cos_hi)) return 0.f;
    const float c = fminf(fmaxf(bcos, -1.0f + 1e-7f), 1.0f - 1e-7f);
    const float beta = acosf(c);
    const float delta = beta - e.theta;
    const float sig_e = delta >= 0.f ? e.sig_plus : e.sig_minus;
    // sigma_pos: grad beta w.r.t. the first hit (inter-crystal leg) and second hit
    const float i01 = 1.0f / fmaxf(d01, 1e-7f);
    const float i12 = 1.0f / fmaxf(e.d12, 1e-7f);
    const float ux = ax * i01, uy = ay * i01, uz = az * i01;
    const float wx = e.vx * i12, wy = e.vy * i12, wz = e.vz * i12;
    const float cb = ux * wx + uy * wy + uz * wz;
    const float sb2 = fmaxf(1.0f - cb * cb, 1e-12f);
    const float jx = (ux - cb * wx) * i12, jy = (uy - cb * wy) * i12, jz = (uz - cb * wz) * i12;
    const float sp2 = (jx * jx * e.s0 + jy * jy * e.s1 + jz * jz * e.s2) / sb2;
    const float sig_pos = sqrtf(fmaxf(sp2, 1e-12f));
    const float sig2 = fmaxf(sig_pos * sig_pos + sig_e * sig_e, 1e-12f);
    const float sinb2 = (1.0f - c) * (1.0f + c);
    return expf(-(delta * delta) / (2.0f * sig2)) * (e.kn - sinb2);
  } else if (MODEL == 2) {
    // simple: exp(-(beta - theta)^2 / (2 sigma_E^2)) / d01^2 with the two-sided sigma_E of the
    // record (the energy resolution propagated through the Compton formula)
    const float bcos = dot / fmaxf(d01 * e.d12, 1e-7f);
    if (WINDOW && (bcos < e.cos_lo || bcos > e.cos_hi)) return 0.f;
    const float c = fminf(fmaxf(bcos, -1.0f + 1e-7f), 1.0f - 1e-7f);
    const float delta = acosf(c) - e.theta;
    const float sig_e = delta >= 0.f ? e.sig_plus : e.sig_minus;
    return expf(-(delta * delta) / (2.0f * sig_e * sig_e)) / fmaxf(d01sq, 1e-14f);
  } else {
    const float beta = acosf(dot / (d01 * e.d12));
    const float delta = beta - e.theta;
    const float sig_e = delta >= 0.f ? e.sig_plus : e.sig_minus;
    const float p = d01 / e.d12;
    const float q = e.s1;
    const float sig_pos = atanf(e.s0 / d01) * sqrtf(1.0f + p * p * (1.0f + q * q) + 2.0f * p * e.s2);
    const float sig = sqrtf(sig_pos * sig_pos + sig_e * sig_e);
    const float sb = sinf(beta);
    return expf(-(delta * delta) / (2.0f * sig * sig)) * (e.kn - sb * sb);
  }
}

// ------------------------------------------------------------------ fast strict evaluation
// The fused forward / back passes evaluate the strict kernel from a staged copy of the record
// whose per-event factors are computed once: the unit second-leg direction w = v12 / d12,
// 1 / d12, and the per-axis position variances divided by d12^2 (the Jacobian of beta in the
// hit positions carries 1 / d12). Per pair: one refined reciprocal square root gives 1 / d01
// and the unit first leg, cos(beta) = (a . w) / d01 serves as both the window test and the
// sigma_pos cosine, sigma_pos^2 is used directly (the formula squares it again), the Gaussian
// exponent takes one quotient, and the quotient and the exponential use the fast hardware forms. The materialised rows and the row
// statistics (event selection) keep the reference-ordered arithmetic of cone_value.
struct alignas(16) ConeFast {
  float p1x, p1y, p1z;
  float wx, wy, wz;       // v12 / max(d12, 1e-7)
  float theta;
  float sig_plus, sig_minus;
  float kn;
  float q0, q1, q2;       // s_k / max(d12, 1e-7)^2
  float cos_lo, cos_hi;
  float pad;
};
static_assert(sizeof(ConeFast) == 64, "staged record layout");

__device__ __forceinline__ ConeFast stage_fast(const ConeEvent& r) {
  ConeFast f;
  const float i12 = 1.0f / fmaxf(r.d12, 1e-7f);
  f.p1x = r.p1x; f.p1y = r.p1y; f.p1z = r.p1z;
  f.wx = r.vx * i12; f.wy = r.vy * i12; f.wz = r.vz * i12;
  f.theta = r.theta;
  f.sig_plus = r.sig_plus;
  f.sig_minus = r.sig_minus;
  f.kn = r.kn;
  f.q0 = r.s0 * i12 * i12; f.q1 = r.s1 * i12 * i12; f.q2 = r.s2 * i12 * i12;
  f.cos_lo = r.cos_lo;
  f.cos_hi = r.cos_hi;
  f.pad = 0.f;
  return f;
}

template <bool WINDOW>
__device__ __forceinline__ float cone_value_fast(const ConeFast& e, float cx, float cy, float cz) {
  const float ax = e.p1x - cx, ay = e.p1y - cy, az = e.p1z - cz;
  const float d2 = fmaxf(fmaf(ax, ax, fmaf(ay, ay, az * az)), 1e-14f);
  // 1 / d01: hardware estimate plus one Newton-Raphson step, r (3 - d2 r^2) / 2
  const float r0 = rsqrtf(d2);
  const float i01 = r0 * fmaf(-0.5f * d2 * r0, r0, 1.5f);
  const float bcos = fmaf(ax, e.wx, fmaf(ay, e.wy, az * e.wz)) * i01;
  if (WINDOW && (bcos < e.cos_lo || bcos > e.cos_hi)) return 0.f;
  const float c = fminf(fmaxf(bcos, -1.0f + 1e-7f), 1.0f - 1e-7f);
  const float delta = acosf(c) - e.theta;
  const float sig_e = delta >= 0.f ? e.sig_plus : e.sig_minus;
  // grad beta: (u01 - cos(beta) w) / d12 per axis, u01 = a / d01
  const float jx = fmaf(-bcos, e.wx, ax * i01);
  const float jy = fmaf(-bcos, e.wy, ay * i01);
  const float jz = fmaf(-bcos, e.wz, az * i01);
  const float sb2 = fmaxf(fmaf(-bcos, bcos, 1.0f), 1e-12f);
  // sigma^2 = max(sigma_E^2 + max(num / sb2, 1e-12), 1e-12) with num / sb2 = sigma_pos^2, carried
  // as sb2 * sigma^2 so the Gaussian exponent needs one quotient
  const float num = fmaf(jx * jx, e.q0, fmaf(jy * jy, e.q1, jz * jz * e.q2));
  const float sig2sb = fmaxf(fmaf(sig_e * sig_e, sb2, fmaxf(num, 1e-12f * sb2)), 1e-12f * sb2);
  const float sinb2 = (1.0f - c) * (1.0f + c);
  return __expf(__fdividef(-(delta * delta) * sb2, 2.0f * sig2sb)) * (e.kn - sinb2);
}

// Record type staged in shared memory and its evaluation: the fast form for the strict model
// in the fused passes, the reference-ordered form otherwise.
template <int MODEL, bool FAST>
struct ConeStage {
  using type = ConeEvent;
  __device__ static ConeEvent stage(const ConeEvent& r) { return r; }
  template <bool WINDOW>
  __device__ static float eval(const ConeEvent& e, float cx, float cy, float cz) {
    return cone_value<MODEL, WINDOW>(e, cx, cy, cz);
  }
};
template <>
struct ConeStage<0, true> {
  using type = ConeFast;
  __device__ static ConeFast stage(const ConeEvent& r) { return stage_fast(r); }
  template <bool WINDOW>
  __device__ static float eval(const ConeFast& e, float cx, float cy, float cz) {
    return cone_value_fast<WINDOW>(e, cx, cy, cz);
  }
};

template <typename TE>
__device__ __forceinline__ float eff_load(const TE* p, int64_t i);
template <>
__device__ __forceinline__ float eff_load<float>(const float* p, int64_t i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float eff_load<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

// ------------------------------------------------------------------ materialised rows
template <int MODEL, typename TE>
__global__ void cone_rows_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                                 const float* __restrict__ coor, int64_t V, const TE* __restrict__ eff,
                                 int64_t ld_eff, float* __restrict__ tc_out, float* __restrict__ t_out) {
  const int64_t i = blockIdx.y;
  if (i >= n_ev) return;
  const ConeEvent e = rec[i];
  const TE* er = eff ? eff + (int64_t)row_id[i] * ld_eff : nullptr;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V; j += (int64_t)gridDim.x * blockDim.x) {
    const float t = cone_value<MODEL, false>(e, coor[3 * j], coor[3 * j + 1], coor[3 * j + 2]);
    if (tc_out) tc_out[i * V + j] = t;
    if (t_out) t_out[i * V + j] = er ? t * eff_load(er, j) : t;
  }
}

// ------------------------------------------------------------------ fused forward
// f[i] = sum_j t_ij eff_ij x_j; optional stats s1[i] = sum t_ij eff_ij, s2[i] = sum (t eff)^2,
// nan[i] = any NaN.
constexpr int kConeThreads = 256;

template <int MODEL, bool WINDOW, int EB, bool STATS, typename TE>
__global__ void __launch_bounds__(kConeThreads)
cone_forward_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                    const float* __restrict__ coor, int64_t V, const float* __restrict__ x,
                    const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ f_out,
                    float* __restrict__ s1_out, float* __restrict__ s2_out, int32_t* __restrict__ nan_out) {
  using Stage = ConeStage<MODEL, !STATS>;
  __shared__ typename Stage::type sev[EB];
  __shared__ int64_t srow[EB];
  __shared__ float red[kConeThreads / 32][EB * (STATS ? 4 : 1)];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t i0 = (int64_t)blockIdx.x * EB;
  if (tid < EB) {
    const int64_t i = i0 + tid < n_ev ? i0 + tid : n_ev - 1;
    sev[tid] = Stage::stage(rec[i]);
    srow[tid] = (int64_t)row_id[i] * ld_eff;
  }
  __syncthreads();
  const int ne = (n_ev - i0) < EB ? (int)(n_ev - i0) : EB;
  float af[EB], a1[EB], a2[EB], an[EB];
#pragma unroll
  for (int e = 0; e < EB; ++e) af[e] = a1[e] = a2[e] = an[e] = 0.f;
  for (int64_t j = tid; j < V; j += kConeThreads) {
    const float cx = coor[3 * j], cy = coor[3 * j + 1], cz = coor[3 * j + 2];
    const float xj = x ? __ldg(x + j) : 0.f;
#pragma unroll
    for (int e = 0; e < EB; ++e) {
      if (e < ne) {
        float t = Stage::template eval<WINDOW>(sev[e], cx, cy, cz);
        if (t != 0.f) {
          t = eff ? t * eff_load(eff + srow[e], j) : t;
          af[e] = fmaf(t, xj, af[e]);
          if (STATS) {
            a1[e] += t;
            a2[e] = fmaf(t, t, a2[e]);
            if (isnan(t)) an[e] = 1.f;
          }
        }
      }
    }
  }
#pragma unroll
  for (int e = 0; e < EB; ++e) {
    const float v = warp_sum(af[e]);
    if (lane == 0) red[warp][e] = v;
    if (STATS) {
      const float v1 = warp_sum(a1[e]);
      const float v2 = warp_sum(a2[e]);
      float vn = an[e];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) vn = fmaxf(vn, __shfl_xor_sync(0xffffffffu, vn, o));
      if (lane == 0) {
        red[warp][EB + e] = v1;
        red[warp][2 * EB + e] = v2;
        red[warp][3 * EB + e] = vn;
      }
    }
  }
  __syncthreads();
  if (tid < ne) {
    float f = 0.f, s1 = 0.f, s2 = 0.f, sn = 0.f;
#pragma unroll
    for (int w = 0; w < kConeThreads / 32; ++w) {
      f += red[w][tid];
      if (STATS) {
        s1 += red[w][EB + tid];
        s2 += red[w][2 * EB + tid];
        sn = fmaxf(sn, red[w][3 * EB + tid]);
      }
    }
    if (f_out) f_out[i0 + tid] = f;
    if (STATS) {
      s1_out[i0 + tid] = s1;
      s2_out[i0 + tid] = s2;
      nan_out[i0 + tid] = sn > 0.f ? 1 : 0;
    }
  }
}

// q[i] = 1 / f[i] (get_weight_compton divides by the forward projection without a floor)
__global__ void cone_ratio_kernel(const float* __restrict__ f, int64_t n, float* __restrict__ q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = 1.0f / f[i];
}

// Batched form: q[i] = 1 / f[i] for events of an instance in [0, n_inst), 0 for padding events
// (event_inst = -1) and, counted, for instance ids out of range.
__global__ void cone_ratio_batch_kernel(const float* __restrict__ f, const int32_t* __restrict__ event_inst,
                                        int64_t n, int n_inst, float* __restrict__ q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int b = event_inst[i];
    if (b >= n_inst) atomicAdd(&g_bad_detector_count, 1u);
    q[i] = (b >= 0 && b < n_inst) ? 1.0f / f[i] : 0.f;
  }
}

// W[b][j] += scale * sum_{c = inst_chunk[b]}^{inst_chunk[b + 1] - 1} part[c][j] (chunks in
// order; chunk offsets clamped to [0, n_chunks], a reversed range counted and skipped).
__global__ void cone_batch_reduce_kernel(const float* __restrict__ part, int64_t ldp, int64_t n_chunks,
                                         const int32_t* __restrict__ inst_chunk, int n_inst, int64_t V, int has_scale,
                                         float scale, float* __restrict__ W, int64_t ldw) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n_inst * V;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / V);
    const int64_t j = t % V;
    int64_t c0 = inst_chunk[b], c1 = inst_chunk[b + 1];
    c0 = c0 < 0 ? 0 : (c0 > n_chunks ? n_chunks : c0);
    c1 = c1 < 0 ? 0 : (c1 > n_chunks ? n_chunks : c1);
    if (c1 < c0) {
      if (j == 0) atomicAdd(&g_bad_detector_count, 1u);
      continue;
    }
    float s = 0.f;
    for (int64_t c = c0; c < c1; ++c) s += part[c * ldp + j];
    float* w = W + (int64_t)b * ldw + j;
    *w = has_scale ? __fadd_rn(*w, __fmul_rn(scale, s)) : __fadd_rn(*w, s);
  }
}

// ------------------------------------------------------------------ fused back projection
// part[chunk][j] = sum_{i in chunk} t_ij eff_ij q_i
constexpr int kBackStage = 128;

template <int MODEL, bool WINDOW, typename TE>
__global__ void __launch_bounds__(kConeThreads)
cone_back_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                 int64_t ev_per_chunk, const float* __restrict__ q, const float* __restrict__ coor, int64_t V,
                 const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ part, int64_t ldp) {
  using Stage = ConeStage<MODEL, true>;
  __shared__ typename Stage::type sev[kBackStage];
  __shared__ int64_t srow[kBackStage];
  __shared__ float sq[kBackStage];
  const int tid = threadIdx.x;
  const int64_t j = (int64_t)blockIdx.x * kConeThreads + tid;
  const int64_t e_begin = (int64_t)blockIdx.y * ev_per_chunk;
  int64_t e_end = e_begin + ev_per_chunk;
  if (e_end > n_ev) e_end = n_ev;
  float cx = 0.f, cy = 0.f, cz = 0.f;
  if (j < V) {
    cx = coor[3 * j];
    cy = coor[3 * j + 1];
    cz = coor[3 * j + 2];
  }
  float acc = 0.f;
  for (int64_t s = e_begin; s < e_end; s += kBackStage) {
    const int n = (e_end - s) < kBackStage ? (int)(e_end - s) : kBackStage;
    __syncthreads();
    if (tid < n) {
      sev[tid] = Stage::stage(rec[s + tid]);
      srow[tid] = (int64_t)row_id[s + tid] * ld_eff;
      sq[tid] = q[s + tid];
    }
    __syncthreads();
    if (j < V) {
      for (int e = 0; e < n; ++e) {
        float t = Stage::template eval<WINDOW>(sev[e], cx, cy, cz);
        if (t != 0.f) {
          t = eff ? t * eff_load(eff + srow[e], j) : t;
          acc = fmaf(t, sq[e], acc);
        }
      }
    }
  }
  if (j < V) part[(int64_t)blockIdx.y * ldp + j] = acc;
}

// ------------------------------------------------------------------ strict pairs (f32x2)
// The strict fused passes evaluate two events per voxel at once: the events' staged fields
// are stored as (event 2k, event 2k + 1) float pairs, and the geometry, the position-variance
// Jacobian, the variance and exponent arithmetic and the Klein-Nishina factor run as packed
// FP32 operations (one f32x2 instruction per two pairs); the reciprocal square root, acos,
// the reciprocal and the exponential stay per lane. Same formulas as cone_value_fast, with
// kn - sin^2(beta) written as (kn - 1) + cos^2(beta).
struct alignas(16) ConePair {
  float2 p1x, p1y, p1z;
  float2 wx, wy, wz;
  float2 ntheta;           // -theta
  float2 knm1;             // kn - 1
  float2 q0, q1, q2;
  float2 sig_plus, sig_minus;
  float2 cos_lo, cos_hi;
  float2 pad;
};
static_assert(sizeof(ConePair) == 128, "pair record layout");

// Writes event r into half h (0: .x, 1: .y) of a staged pair.
__device__ __forceinline__ void stage_pair_half(ConePair* pr, int h, const ConeEvent& r) {
  const ConeFast f = stage_fast(r);
  float* d = reinterpret_cast<float*>(pr) + h;
  const float v[16] = {f.p1x, f.p1y, f.p1z, f.wx, f.wy, f.wz, -f.theta, f.kn - 1.0f,
                       f.q0, f.q1, f.q2, f.sig_plus, f.sig_minus, f.cos_lo, f.cos_hi, 0.f};
#pragma unroll
  for (int k = 0; k < 16; ++k) d[2 * k] = v[k];
}

__device__ __forceinline__ float ex2_approx(float z) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(z));
  return r;
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

// arccos of two cosines (|c| < 1) by the rational-free approximation of Abramowitz & Stegun,
// Handbook of Mathematical Functions, 4.4.46 (after Hastings): acos(x) = sqrt(1 - x) P7(x) on
// [0, 1], |error| <= 2e-8 in exact arithmetic, and acos(x) = pi - acos(-x) below 0. The
// square root is 1 - |x| times its reciprocal square root refined by one Newton step, in
// packed f32x2 arithmetic (float32 evaluation error: a few 1e-7 rad; checked against acosf by
// the cone tests through the fused-versus-stored weights).
__device__ __forceinline__ float2 acos2_as4446(float2 c) {
  const float2 a = make_float2(fabsf(c.x), fabsf(c.y));
  float2 p = f2(-0.0012624911f);
  p = __ffma2_rn(p, a, f2(0.0066700901f));
  p = __ffma2_rn(p, a, f2(-0.0170881256f));
  p = __ffma2_rn(p, a, f2(0.0308918810f));
  p = __ffma2_rn(p, a, f2(-0.0501743046f));
  p = __ffma2_rn(p, a, f2(0.0889789874f));
  p = __ffma2_rn(p, a, f2(-0.2145988016f));
  p = __ffma2_rn(p, a, f2(1.5707963050f));
  const float2 om = __ffma2_rn(a, f2(-1.0f), f2(1.0f));  // 1 - |x| (exact for |x| >= 1/2)
  const float2 r = make_float2(rsqrtf(om.x), rsqrtf(om.y));
  float2 sq = __fmul2_rn(om, r);
  const float2 err = __ffma2_rn(__fmul2_rn(sq, f2(-1.0f)), sq, om);  // om - sq^2
  sq = __ffma2_rn(err, __fmul2_rn(r, f2(0.5f)), sq);
  const float2 v = __fmul2_rn(sq, p);
  const float2 w = __fadd2_rn(f2(3.14159265358979f), __fmul2_rn(v, f2(-1.0f)));  // pi - v
  return make_float2(c.x < 0.f ? w.x : v.x, c.y < 0.f ? w.y : v.y);
}

// t for the two events of a staged pair at one voxel (ncx.. = minus the voxel centre).
template <bool WINDOW>
__device__ __forceinline__ float2 cone_pair_fast(const ConePair& e, float2 ncx, float2 ncy, float2 ncz) {
  const float2 ax = __fadd2_rn(e.p1x, ncx), ay = __fadd2_rn(e.p1y, ncy), az = __fadd2_rn(e.p1z, ncz);
  float2 d2 = __ffma2_rn(ax, ax, __ffma2_rn(ay, ay, __fmul2_rn(az, az)));
  d2.x = fmaxf(d2.x, 1e-14f);
  d2.y = fmaxf(d2.y, 1e-14f);
  const float2 r0 = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
  // 1 / d01: one Newton-Raphson step, r (3 - d2 r^2) / 2
  const float2 h = __fmul2_rn(__fmul2_rn(d2, f2(-0.5f)), r0);
  const float2 i01 = __fmul2_rn(r0, __ffma2_rn(h, r0, f2(1.5f)));
  const float2 dotw = __ffma2_rn(ax, e.wx, __ffma2_rn(ay, e.wy, __fmul2_rn(az, e.wz)));
  const float2 bcos = __fmul2_rn(dotw, i01);
  bool in0 = true, in1 = true;
  if (WINDOW) {
    in0 = !(bcos.x < e.cos_lo.x || bcos.x > e.cos_hi.x);
    in1 = !(bcos.y < e.cos_lo.y || bcos.y > e.cos_hi.y);
    if (!(in0 || in1)) return make_float2(0.f, 0.f);
  }
  const float2 c = make_float2(fminf(fmaxf(bcos.x, -1.0f + 1e-7f), 1.0f - 1e-7f),
                               fminf(fmaxf(bcos.y, -1.0f + 1e-7f), 1.0f - 1e-7f));
  const float2 delta = __fadd2_rn(acos2_as4446(c), e.ntheta);
  const float2 sig_e = make_float2(delta.x >= 0.f ? e.sig_plus.x : e.sig_minus.x,
                                   delta.y >= 0.f ? e.sig_plus.y : e.sig_minus.y);
  // grad beta per axis: (u01 - cos(beta) w) / d12 = (a - (a . w) w) / (d01 d12); the 1 / d12^2 is
  // in q, the 1 / d01^2 is applied once to the sum
  const float2 ndw = __fmul2_rn(dotw, f2(-1.0f));
  const float2 jx = __ffma2_rn(ndw, e.wx, ax);
  const float2 jy = __ffma2_rn(ndw, e.wy, ay);
  const float2 jz = __ffma2_rn(ndw, e.wz, az);
  float2 sb2 = __ffma2_rn(__fmul2_rn(bcos, f2(-1.0f)), bcos, f2(1.0f));
  sb2.x = fmaxf(sb2.x, 1e-12f);
  sb2.y = fmaxf(sb2.y, 1e-12f);
  const float2 num = __fmul2_rn(__ffma2_rn(__fmul2_rn(jx, jx), e.q0,
                                           __ffma2_rn(__fmul2_rn(jy, jy), e.q1, __fmul2_rn(__fmul2_rn(jz, jz), e.q2))),
                                __fmul2_rn(i01, i01));
  // sb2 * sigma^2 = max(sigma_E^2 sb2 + max(num, 1e-12 sb2), 1e-12 sb2)
  // (the outer max is implied: sigma_E^2 sb2 >= 0 and the addend is >= 1e-12 sb2, and a
  // rounded sum of the two cannot fall below the addend)
  const float2 tiny = __fmul2_rn(sb2, f2(1e-12f));
  const float2 s2 =
      __ffma2_rn(__fmul2_rn(sig_e, sig_e), sb2, make_float2(fmaxf(num.x, tiny.x), fmaxf(num.y, tiny.y)));
  // exp(-delta^2 / (2 sigma^2)) = 2^(-log2(e) / 2 * delta^2 sb2 / (sb2 sigma^2))
  const float2 nd = __fmul2_rn(__fmul2_rn(delta, delta), sb2);
  const float2 z = __fmul2_rn(__fmul2_rn(nd, make_float2(__fdividef(1.0f, s2.x), __fdividef(1.0f, s2.y))),
                              f2(-0.72134752044448170f));
  float2 t = __fmul2_rn(make_float2(ex2_approx(z.x), ex2_approx(z.y)), __ffma2_rn(c, c, e.knm1));
  if (WINDOW) {
    if (!in0) t.x = 0.f;
    if (!in1) t.y = 0.f;
  }
  return t;
}

// f[i] = sum_j t_ij eff_ij x_j for the strict model, 16 events (8 pairs) per CTA.
// BATCH: several instances' events in one launch; every 16-event block belongs to one
// instance (block_inst[block]), whose image is x + instance * ldx; a block whose instance is
// outside [0, n_inst) is skipped (f = 0) and counted.
template <bool WINDOW, typename TE, bool BATCH = false>
__global__ void __launch_bounds__(kConeThreads, 5)
cone_forward_pair_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                         const float* __restrict__ coor, int64_t V, const float* __restrict__ x,
                         const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ f_out,
                         const int32_t* __restrict__ block_inst, int64_t ldx, int n_inst) {
  constexpr int EB = 16, NP = EB / 2;
  __shared__ ConePair sev[NP];
  __shared__ int64_t srow[EB];
  __shared__ float red[kConeThreads / 32][EB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t i0 = (int64_t)blockIdx.x * EB;
  int64_t v_end = V;
  if (BATCH) {
    const int b = block_inst[blockIdx.x];
    if (b < 0 || b >= n_inst) {
      if (tid == 0) atomicAdd(&g_bad_detector_count, 1u);
      v_end = 0;  // no voxel: f = 0
    } else {
      x += (int64_t)b * ldx;
    }
  }
  if (tid < EB) {
    const int64_t i = i0 + tid < n_ev ? i0 + tid : n_ev - 1;  // padding repeats a valid event
    stage_pair_half(&sev[tid >> 1], tid & 1, rec[i]);
    srow[tid] = (int64_t)row_id[i] * ld_eff;
  }
  __syncthreads();
  const int ne = (n_ev - i0) < EB ? (int)(n_ev - i0) : EB;
  const int np = (ne + 1) >> 1;
  float2 af[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) af[k] = make_float2(0.f, 0.f);
  for (int64_t j = tid; j < v_end; j += kConeThreads) {
    const float2 ncx = f2(-coor[3 * j]), ncy = f2(-coor[3 * j + 1]), ncz = f2(-coor[3 * j + 2]);
    const float2 xj = f2(x ? __ldg(x + j) : 0.f);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      if (k < np) {
        float2 t = cone_pair_fast<WINDOW>(sev[k], ncx, ncy, ncz);
        if constexpr (WINDOW) {
          // pairs outside the window skip their efficiency load
          if (t.x != 0.f || t.y != 0.f) {
            if (eff) {
              t.x = t.x != 0.f ? t.x * eff_load(eff + srow[2 * k], j) : 0.f;
              t.y = t.y != 0.f ? t.y * eff_load(eff + srow[2 * k + 1], j) : 0.f;
            }
            af[k] = __ffma2_rn(t, xj, af[k]);
          }
        } else {
          if (eff) t = __fmul2_rn(t, make_float2(eff_load(eff + srow[2 * k], j), eff_load(eff + srow[2 * k + 1], j)));
          af[k] = __ffma2_rn(t, xj, af[k]);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const float v0 = warp_sum(af[k].x);
    const float v1 = warp_sum(af[k].y);
    if (lane == 0) {
      red[warp][2 * k] = v0;
      red[warp][2 * k + 1] = v1;
    }
  }
  __syncthreads();
  if (tid < ne) {
    float f = 0.f;
#pragma unroll
    for (int w = 0; w < kConeThreads / 32; ++w) f += red[w][tid];
    if (f_out) f_out[i0 + tid] = f;
  }
}

// part[chunk][j] = sum_{i in chunk} t_ij eff_ij q_i for the strict model, events in pairs.
// BATCH: chunk c holds events chunk_range[c] .. chunk_range[c + 1] (clamped to [0, n_ev]).
template <bool WINDOW, typename TE, bool BATCH = false>
__global__ void __launch_bounds__(kConeThreads, 8)
cone_back_pair_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                      int64_t ev_per_chunk, const float* __restrict__ q, const float* __restrict__ coor, int64_t V,
                      const TE* __restrict__ eff, int64_t ld_eff, float* __restrict__ part, int64_t ldp,
                      const int64_t* __restrict__ chunk_range) {
  __shared__ ConePair sev[kBackStage / 2];
  __shared__ int64_t srow[kBackStage];
  __shared__ float sq[kBackStage];
  const int tid = threadIdx.x;
  const int64_t j = (int64_t)blockIdx.x * kConeThreads + tid;
  int64_t e_begin, e_end;
  if (BATCH) {
    e_begin = chunk_range[blockIdx.y];
    e_end = chunk_range[blockIdx.y + 1];
    e_begin = e_begin < 0 ? 0 : (e_begin > n_ev ? n_ev : e_begin);
    e_end = e_end < e_begin ? e_begin : (e_end > n_ev ? n_ev : e_end);
  } else {
    e_begin = (int64_t)blockIdx.y * ev_per_chunk;
    e_end = e_begin + ev_per_chunk;
    if (e_end > n_ev) e_end = n_ev;
  }
  float2 ncx = f2(0.f), ncy = f2(0.f), ncz = f2(0.f);
  if (j < V) {
    ncx = f2(-coor[3 * j]);
    ncy = f2(-coor[3 * j + 1]);
    ncz = f2(-coor[3 * j + 2]);
  }
  float2 acc = make_float2(0.f, 0.f);
  for (int64_t s = e_begin; s < e_end; s += kBackStage) {
    const int n = (e_end - s) < kBackStage ? (int)(e_end - s) : kBackStage;
    __syncthreads();
    if (tid < n) {
      stage_pair_half(&sev[tid >> 1], tid & 1, rec[s + tid]);
      srow[tid] = (int64_t)row_id[s + tid] * ld_eff;
      sq[tid] = q[s + tid];
    } else if (tid == n && (n & 1)) {
      // odd count: the pair's second half repeats event s with a zero ratio
      stage_pair_half(&sev[tid >> 1], 1, rec[s]);
      srow[tid] = (int64_t)row_id[s] * ld_eff;
      sq[tid] = 0.f;
    }
    __syncthreads();
    if (j < V) {
      const int np = (n + 1) >> 1;
      for (int k = 0; k < np; ++k) {
        float2 t = cone_pair_fast<WINDOW>(sev[k], ncx, ncy, ncz);
        if constexpr (WINDOW) {
          if (t.x != 0.f || t.y != 0.f) {
            if (eff) {
              t.x = t.x != 0.f ? t.x * eff_load(eff + srow[2 * k], j) : 0.f;
              t.y = t.y != 0.f ? t.y * eff_load(eff + srow[2 * k + 1], j) : 0.f;
            }
            acc = __ffma2_rn(t, make_float2(sq[2 * k], sq[2 * k + 1]), acc);
          }
        } else {
          if (eff) t = __fmul2_rn(t, make_float2(eff_load(eff + srow[2 * k], j), eff_load(eff + srow[2 * k + 1], j)));
          acc = __ffma2_rn(t, make_float2(sq[2 * k], sq[2 * k + 1]), acc);
        }
      }
    }
  }
  if (j < V) part[(int64_t)blockIdx.y * ldp + j] = acc.x + acc.y;
}

// ------------------------------------------------------------------ FP64 evaluation
// Reference-grade projector halves for gradient checks: the strict kernel of
// process_list_plane_strict.py:201-228 evaluated in double from the same records (no window,
// no staged factors), sums in double. Not a hot path: one CTA per event forward, one thread
// per voxel back.
__device__ __forceinline__ double cone_strict_f64(const ConeEvent& e, double cx, double cy, double cz) {
  const double ax = (double)e.p1x - cx, ay = (double)e.p1y - cy, az = (double)e.p1z - cz;
  const double vx = e.vx, vy = e.vy, vz = e.vz, d12 = e.d12;
  const double dot = ax * vx + ay * vy + az * vz;
  const double d01 = sqrt(ax * ax + ay * ay + az * az);
  const double bcos = dot / fmax(d01 * d12, 1e-7);
  const double c = fmin(fmax(bcos, -1.0 + 1e-7), 1.0 - 1e-7);
  const double delta = acos(c) - (double)e.theta;
  const double sig_e = delta >= 0.0 ? (double)e.sig_plus : (double)e.sig_minus;
  const double i01 = 1.0 / fmax(d01, 1e-7), i12 = 1.0 / fmax(d12, 1e-7);
  const double ux = ax * i01, uy = ay * i01, uz = az * i01;
  const double wx = vx * i12, wy = vy * i12, wz = vz * i12;
  const double cb = ux * wx + uy * wy + uz * wz;
  const double sb2 = fmax(1.0 - cb * cb, 1e-12);
  const double jx = (ux - cb * wx) * i12, jy = (uy - cb * wy) * i12, jz = (uz - cb * wz) * i12;
  const double sp2 = (jx * jx * e.s0 + jy * jy * e.s1 + jz * jz * e.s2) / sb2;
  const double sig_pos = sqrt(fmax(sp2, 1e-12));
  const double sig2 = fmax(sig_pos * sig_pos + sig_e * sig_e, 1e-12);
  return exp(-(delta * delta) / (2.0 * sig2)) * ((double)e.kn - (1.0 - c) * (1.0 + c));
}

template <typename TE>
__device__ __forceinline__ double eff_f64(const TE* p, int64_t i) {
  return (double)eff_load(p, i);
}

// f[i] = sum_j t_ij eff_ij x_j
template <typename TE>
__global__ void __launch_bounds__(256)
cone_forward_f64_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                        const float* __restrict__ coor, int64_t V, const double* __restrict__ x,
                        const TE* __restrict__ eff, int64_t ld_eff, double* __restrict__ f_out) {
  __shared__ double red[8];
  for (int64_t i = blockIdx.x; i < n_ev; i += gridDim.x) {
    const ConeEvent e = rec[i];
    const TE* er = eff ? eff + (int64_t)row_id[i] * ld_eff : nullptr;
    double acc = 0.0;
    for (int64_t j = threadIdx.x; j < V; j += blockDim.x) {
      double t = cone_strict_f64(e, coor[3 * j], coor[3 * j + 1], coor[3 * j + 2]);
      if (er) t *= eff_f64(er, j);
      acc += t * x[j];
    }
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double f = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) f += red[w];
      f_out[i] = f;
    }
    __syncthreads();
  }
}

// weight[j] += scale * sum_i t_ij eff_ij g_i
template <typename TE>
__global__ void __launch_bounds__(256)
cone_back_f64_kernel(const ConeEvent* __restrict__ rec, const int32_t* __restrict__ row_id, int64_t n_ev,
                     const float* __restrict__ coor, int64_t V, const double* __restrict__ g,
                     const TE* __restrict__ eff, int64_t ld_eff, double scale, double* __restrict__ weight) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < V; j += (int64_t)gridDim.x * blockDim.x) {
    const double cx = coor[3 * j], cy = coor[3 * j + 1], cz = coor[3 * j + 2];
    double acc = 0.0;
    for (int64_t i = 0; i < n_ev; ++i) {
      double t = cone_strict_f64(rec[i], cx, cy, cz);
      if (eff) t *= eff_f64(eff + (int64_t)row_id[i] * ld_eff, j);
      acc += t * g[i];
    }
    weight[j] += scale * acc;
  }
}

// ------------------------------------------------------------------ host planning
struct ConePlan {
  int64_t chunks;
  int64_t ev_per_chunk;
  int64_t ldp;
  int64_t ldx;
  size_t ws_bytes;
};

static ConePlan plan_cone(int64_t n_ev, int64_t V) {
  ConePlan p{};
  const int64_t tiles = (V + kConeThreads - 1) / kConeThreads;
  const int64_t target = 2432;  // back-pass CTAs: 16 x 152 SMs
  int64_t chunks = (target + tiles - 1) / (tiles > 0 ? tiles : 1);
  const int64_t max_chunks = (n_ev + 63) / 64;  // >= 64 events per chunk
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks < 1) chunks = 1;
  p.ev_per_chunk = (n_ev + chunks - 1) / chunks;
  if (p.ev_per_chunk < 1) p.ev_per_chunk = 1;
  p.chunks = (n_ev + p.ev_per_chunk - 1) / p.ev_per_chunk;
  if (p.chunks < 1) p.chunks = 1;
  p.ldp = (int64_t)align_up((size_t)(V > 0 ? V : 1), 8);
  p.ldx = p.ldp;
  size_t b = 0;
  b += align_up((size_t)p.ldx * sizeof(float), 256);                       // rotated image
  b += align_up((size_t)(n_ev > 0 ? n_ev : 1) * sizeof(float), 256) * 2;  // f, q
  b += align_up((size_t)p.chunks * p.ldp * sizeof(float), 256);            // partials
  p.ws_bytes = b + 256;
  return p;
}

template <int MODEL, bool WINDOW, typename TE>
static int launch_cone_weight(const ConeEvent* rec, const int32_t* rid, int64_t n_ev, const float* coor, int64_t V,
                              const float* x, const TE* eff, int64_t ld_eff, float* f, float* q, float* part,
                              const ConePlan& p, cudaStream_t st, int stage = 0) {
  // stage 0: forward, ratio, back (the weight); 1: forward only (f); 2: back-project q
  constexpr int EB = 16;
  if (stage != 2) {
    const unsigned fgrid = (unsigned)((n_ev + EB - 1) / EB);
    if (MODEL == 0)
      JSCC_TIMED("cone_forward", st,
                 (cone_forward_pair_kernel<WINDOW, TE><<<fgrid, kConeThreads, 0, st>>>(rec, rid, n_ev, coor, V, x,
                                                                                       eff, ld_eff, f, nullptr, 0,
                                                                                       0)));
    else
      JSCC_TIMED("cone_forward", st,
                 (cone_forward_kernel<MODEL, WINDOW, EB, false, TE><<<fgrid, kConeThreads, 0, st>>>(
                     rec, rid, n_ev, coor, V, x, eff, ld_eff, f, nullptr, nullptr, nullptr)));
    JSCC_LAUNCH_CHECK();
    if (stage == 1) return JSCC_OK;
    int64_t rb = (n_ev + 255) / 256;
    if (rb > 4096) rb = 4096;
    JSCC_TIMED("cone_ratio", st, (cone_ratio_kernel<<<(unsigned)rb, 256, 0, st>>>(f, n_ev, q)));
    JSCC_LAUNCH_CHECK();
  }
  dim3 bgrid((unsigned)((V + kConeThreads - 1) / kConeThreads), (unsigned)p.chunks);
  if (MODEL == 0)
    JSCC_TIMED("cone_back", st,
               (cone_back_pair_kernel<WINDOW, TE><<<bgrid, kConeThreads, 0, st>>>(
                   rec, rid, n_ev, p.ev_per_chunk, q, coor, V, eff, ld_eff, part, p.ldp, nullptr)));
  else
    JSCC_TIMED("cone_back", st,
               (cone_back_kernel<MODEL, WINDOW, TE><<<bgrid, kConeThreads, 0, st>>>(
                   rec, rid, n_ev, p.ev_per_chunk, q, coor, V, eff, ld_eff, part, p.ldp)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

}  // namespace jscc

using namespace jscc;

extern "C" {

int jscc_compton_event_prep(const float* list, int64_t ld_list, int64_t n_events, const float* det_pos,
                            const float* sig1_sq, const float* sig2_sq, int64_t n_det, float e0,
                            float ene_resolution, float thr_max, float thr_min, float thr_sum, int32_t model,
                            int32_t theta_fp64, float window_sigmas, float delta_r1, float delta_r2,
                            uint8_t* keep, float* records, int32_t* row_id, void* stream) {
  JSCC_REQUIRE(n_events >= 0 && n_det >= 0, "jscc_compton_event_prep: negative size");
  JSCC_REQUIRE(model == JSCC_CONE_STRICT || model == JSCC_CONE_LEGACY || model == JSCC_CONE_SIMPLE,
               "jscc_compton_event_prep: bad model %d",
               model);
  if (n_events == 0) return JSCC_OK;
  JSCC_REQUIRE(list && det_pos && keep && records && row_id, "jscc_compton_event_prep: null pointer argument");
  JSCC_REQUIRE(model == JSCC_CONE_LEGACY || (sig1_sq && sig2_sq),
               "jscc_compton_event_prep: strict model needs the position-variance tables");
  JSCC_REQUIRE(ld_list >= 4, "jscc_compton_event_prep: ld_list < 4");
  JSCC_REQUIRE(reinterpret_cast<uintptr_t>(records) % 16 == 0, "jscc_compton_event_prep: records not 16-byte aligned");
  cudaStream_t st = as_stream(stream);
  int64_t blocks = (n_events + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  JSCC_TIMED("compton_event_prep", st,
             (compton_event_prep_kernel<<<(unsigned)blocks, 256, 0, st>>>(
                 list, ld_list, n_events, det_pos, sig1_sq, sig2_sq, n_det, e0, ene_resolution, thr_max, thr_min,
                 thr_sum, model, theta_fp64, window_sigmas, delta_r1, delta_r2, keep,
                 reinterpret_cast<ConeEvent*>(records), row_id)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_compton_cone_rows(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor, int64_t V,
                           int32_t model, const void* eff, int32_t eff_dtype, int64_t ld_eff, float* t_compton,
                           float* t, void* stream) {
  JSCC_REQUIRE(n_ev >= 0 && V >= 0, "jscc_compton_cone_rows: negative size");
  JSCC_REQUIRE(model == JSCC_CONE_STRICT || model == JSCC_CONE_LEGACY || model == JSCC_CONE_SIMPLE,
               "jscc_compton_cone_rows: bad model");
  JSCC_REQUIRE(eff_dtype == JSCC_DTYPE_F32 || eff_dtype == JSCC_DTYPE_BF16, "jscc_compton_cone_rows: bad dtype");
  if (n_ev == 0 || V == 0) return JSCC_OK;
  JSCC_REQUIRE(records && coor && (t_compton || t), "jscc_compton_cone_rows: null pointer argument");
  JSCC_REQUIRE(!eff || (row_id && ld_eff >= V), "jscc_compton_cone_rows: efficiency rows need row ids and ld >= V");
  JSCC_REQUIRE(n_ev <= 65535, "jscc_compton_cone_rows: at most 65,535 events per call (got %lld)", (long long)n_ev);
  cudaStream_t st = as_stream(stream);
  const ConeEvent* rec = reinterpret_cast<const ConeEvent*>(records);
  int64_t bx = (V + 255) / 256;
  if (bx > 64) bx = 64;
  dim3 grid((unsigned)bx, (unsigned)n_ev);
  if (eff_dtype == JSCC_DTYPE_F32) {
    const float* e = static_cast<const float*>(eff);
    if (model == JSCC_CONE_STRICT)
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<0, float><<<grid, 256, 0, st>>>(rec, row_id, n_ev, coor, V, e,
                                                                                        ld_eff, t_compton, t)));
    else if (model == JSCC_CONE_SIMPLE)
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<2, float><<<grid, 256, 0, st>>>(rec, row_id, n_ev, coor, V, e,
                                                                                        ld_eff, t_compton, t)));
    else
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<1, float><<<grid, 256, 0, st>>>(rec, row_id, n_ev, coor, V, e,
                                                                                        ld_eff, t_compton, t)));
  } else {
    const __nv_bfloat16* e = static_cast<const __nv_bfloat16*>(eff);
    if (model == JSCC_CONE_STRICT)
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<0, __nv_bfloat16><<<grid, 256, 0, st>>>(
                                      rec, row_id, n_ev, coor, V, e, ld_eff, t_compton, t)));
    else if (model == JSCC_CONE_SIMPLE)
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<2, __nv_bfloat16><<<grid, 256, 0, st>>>(
                                      rec, row_id, n_ev, coor, V, e, ld_eff, t_compton, t)));
    else
      JSCC_TIMED("cone_rows", st, (cone_rows_kernel<1, __nv_bfloat16><<<grid, 256, 0, st>>>(
                                      rec, row_id, n_ev, coor, V, e, ld_eff, t_compton, t)));
  }
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_compton_row_stats(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor, int64_t V,
                           int32_t model, int32_t use_window, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                           float* s1, float* s2, int32_t* nan_flag, void* stream) {
  JSCC_REQUIRE(n_ev >= 0 && V >= 0, "jscc_compton_row_stats: negative size");
  JSCC_REQUIRE(model == JSCC_CONE_STRICT || model == JSCC_CONE_LEGACY || model == JSCC_CONE_SIMPLE,
               "jscc_compton_row_stats: bad model");
  JSCC_REQUIRE(eff_dtype == JSCC_DTYPE_F32 || eff_dtype == JSCC_DTYPE_BF16, "jscc_compton_row_stats: bad dtype");
  if (n_ev == 0) return JSCC_OK;
  JSCC_REQUIRE(records && coor && s1 && s2 && nan_flag, "jscc_compton_row_stats: null pointer argument");
  JSCC_REQUIRE(!eff || (row_id && ld_eff >= V), "jscc_compton_row_stats: efficiency rows need row ids and ld >= V");
  cudaStream_t st = as_stream(stream);
  const ConeEvent* rec = reinterpret_cast<const ConeEvent*>(records);
  constexpr int EB = 8;
  const unsigned grid = (unsigned)((n_ev + EB - 1) / EB);
#define JSCC_STATS_LAUNCH(M, W, TE)                                                                            \
  JSCC_TIMED("cone_row_stats", st,                                                                             \
             (cone_forward_kernel<M, W, EB, true, TE><<<grid, kConeThreads, 0, st>>>(                          \
                 rec, row_id, n_ev, coor, V, nullptr, static_cast<const TE*>(eff), ld_eff, nullptr, s1, s2,    \
                 nan_flag)))
  if (eff_dtype == JSCC_DTYPE_F32) {
    if (model == JSCC_CONE_LEGACY) JSCC_STATS_LAUNCH(1, false, float);
    else if (model == JSCC_CONE_SIMPLE) JSCC_STATS_LAUNCH(2, false, float);
    else if (use_window) JSCC_STATS_LAUNCH(0, true, float);
    else JSCC_STATS_LAUNCH(0, false, float);
  } else {
    if (model == JSCC_CONE_LEGACY) JSCC_STATS_LAUNCH(1, false, __nv_bfloat16);
    else if (model == JSCC_CONE_SIMPLE) JSCC_STATS_LAUNCH(2, false, __nv_bfloat16);
    else if (use_window) JSCC_STATS_LAUNCH(0, true, __nv_bfloat16);
    else JSCC_STATS_LAUNCH(0, false, __nv_bfloat16);
  }
#undef JSCC_STATS_LAUNCH
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

size_t jscc_compton_weight_workspace_bytes(int64_t n_ev, int64_t n_vox) { return plan_cone(n_ev, n_vox).ws_bytes; }

// The weight and its two halves (the differentiable projector's forward and backward):
// stage 0: weight += scale * rotinv(T^T (1 / T rot(img))); 1: f_out[i] = sum_j t_ij rot(img)_j;
// 2: weight += scale * rotinv(T^T g).
static int compton_stage_entry(const char* what, int stage, const float* records, const int32_t* row_id,
                               int64_t n_ev, const float* coor, int64_t n_vox, int32_t model, int32_t use_window,
                               const void* eff, int32_t eff_dtype, int64_t ld_eff, const float* img,
                               const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, const float* g,
                               float* f_out, float scale, float* weight, void* workspace, size_t workspace_bytes,
                               void* stream) {
  JSCC_REQUIRE(n_ev >= 0 && n_vox >= 0, "%s: negative size", what);
  JSCC_REQUIRE(model == JSCC_CONE_STRICT || model == JSCC_CONE_LEGACY || model == JSCC_CONE_SIMPLE,
               "%s: bad model", what);
  JSCC_REQUIRE(eff_dtype == JSCC_DTYPE_F32 || eff_dtype == JSCC_DTYPE_BF16, "%s: bad dtype", what);
  if (n_ev == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(records && coor, "%s: null pointer argument", what);
  JSCC_REQUIRE(stage == 2 || img, "%s: null image", what);
  JSCC_REQUIRE(stage != 1 || f_out, "%s: null output", what);
  JSCC_REQUIRE(stage == 1 || weight, "%s: null weight", what);
  JSCC_REQUIRE(stage != 2 || g, "%s: null input", what);
  JSCC_REQUIRE(!eff || (row_id && ld_eff >= n_vox), "%s: efficiency rows need row ids, ld >= V", what);
  JSCC_REQUIRE(stage != 0 || (rotmat == nullptr) == (rotmat_inv == nullptr), "%s: give both rotation tables", what);
  const ConePlan p = plan_cone(n_ev, n_vox);
  JSCC_REQUIRE(workspace && workspace_bytes >= p.ws_bytes, "%s: workspace too small (%zu < %zu)", what,
               workspace_bytes, p.ws_bytes);
  Carver cv(workspace, workspace_bytes);
  float* xr = cv.take<float>((size_t)p.ldx);
  float* f = cv.take<float>((size_t)n_ev);
  float* q = cv.take<float>((size_t)n_ev);
  float* part = cv.take<float>((size_t)p.chunks * p.ldp);
  JSCC_REQUIRE(cv.ok(), "%s: workspace carve overflow", what);
  if (stage == 1) f = f_out;
  if (stage == 2) q = const_cast<float*>(g);  // read only by the back kernel
  cudaStream_t st = as_stream(stream);
  const ConeEvent* rec = reinterpret_cast<const ConeEvent*>(records);
  const float* x = img;
  if (rotmat && stage != 2) {
    int64_t blocks = (n_vox + 255) / 256;
    if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
    JSCC_TIMED("sc_gather_rot", st,
               (sc_gather_rot_kernel<<<(unsigned)blocks, 256, 0, st>>>(img, rotmat, ld_rot, 0, 1, n_vox, p.ldx, xr)));
    JSCC_LAUNCH_CHECK();
    x = xr;
  }
  int rc;
  const bool win = use_window != 0 && model == JSCC_CONE_STRICT;
  if (eff_dtype == JSCC_DTYPE_F32) {
    const float* e = static_cast<const float*>(eff);
    if (model == JSCC_CONE_LEGACY)
      rc = launch_cone_weight<1, false, float>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p, st, stage);
    else if (model == JSCC_CONE_SIMPLE)
      rc = launch_cone_weight<2, false, float>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p, st, stage);
    else if (win)
      rc = launch_cone_weight<0, true, float>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p, st, stage);
    else
      rc = launch_cone_weight<0, false, float>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p, st, stage);
  } else {
    const __nv_bfloat16* e = static_cast<const __nv_bfloat16*>(eff);
    if (model == JSCC_CONE_LEGACY)
      rc = launch_cone_weight<1, false, __nv_bfloat16>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p,
                                                       st, stage);
    else if (model == JSCC_CONE_SIMPLE)
      rc = launch_cone_weight<2, false, __nv_bfloat16>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p,
                                                       st, stage);
    else if (win)
      rc = launch_cone_weight<0, true, __nv_bfloat16>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p,
                                                      st, stage);
    else
      rc = launch_cone_weight<0, false, __nv_bfloat16>(rec, row_id, n_ev, coor, n_vox, x, e, ld_eff, f, q, part, p,
                                                       st, stage);
  }
  if (rc != JSCC_OK || stage == 1) return rc;
  int64_t blocks = (n_vox + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  const int has_scale = scale != 1.0f;
  JSCC_TIMED("sc_reduce_scatter", st,
             (sc_reduce_scatter_kernel<<<(unsigned)blocks, 256, 0, st>>>(part, p.ldp, (int)p.chunks, 1, 1, rotmat_inv,
                                                                          ld_rot, 0, n_vox, has_scale, scale,
                                                                          weight)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_compton_weight(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor, int64_t n_vox,
                        int32_t model, int32_t use_window, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                        const float* img, const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot,
                        float scale, float* weight, void* workspace, size_t workspace_bytes, void* stream) {
  return compton_stage_entry("jscc_compton_weight", 0, records, row_id, n_ev, coor, n_vox, model, use_window, eff,
                             eff_dtype, ld_eff, img, rotmat, rotmat_inv, ld_rot, nullptr, nullptr, scale, weight,
                             workspace, workspace_bytes, stream);
}

size_t jscc_compton_batch_workspace_bytes(int64_t n_ev, int64_t n_chunks, int64_t n_vox) {
  if (n_ev < 0 || n_chunks < 0 || n_vox < 0) return 0;
  const int64_t ldp = (int64_t)align_up((size_t)(n_vox > 0 ? n_vox : 1), 8);
  return align_up((size_t)(n_ev > 0 ? n_ev : 1) * sizeof(float), 256) * 2 +
         align_up((size_t)(n_chunks > 0 ? n_chunks : 1) * ldp * sizeof(float), 256) + 256;
}

int jscc_compton_weight_batched(const float* records, const int32_t* row_id, int64_t n_ev, const int32_t* event_inst,
                                const int32_t* block_inst, const int64_t* chunk_range, const int32_t* inst_chunk,
                                int64_t n_chunks, int32_t n_inst, const float* coor, int64_t n_vox, const void* eff,
                                int32_t eff_dtype, int64_t ld_eff, const float* X, int64_t ldx, float scale, float* W,
                                int64_t ldw, void* workspace, size_t workspace_bytes, void* stream) {
  const char* what = "jscc_compton_weight_batched";
  JSCC_REQUIRE(n_ev >= 0 && n_vox >= 0 && n_chunks >= 0 && n_inst >= 0, "%s: negative size", what);
  JSCC_REQUIRE(eff_dtype == JSCC_DTYPE_F32 || eff_dtype == JSCC_DTYPE_BF16, "%s: bad dtype", what);
  if (n_ev == 0 || n_vox == 0 || n_inst == 0 || n_chunks == 0) return JSCC_OK;
  JSCC_REQUIRE(n_ev % 16 == 0, "%s: n_ev (%lld) must be a multiple of 16 (pad each instance)", what,
               (long long)n_ev);
  JSCC_REQUIRE(records && coor && event_inst && block_inst && chunk_range && inst_chunk && X && W,
               "%s: null pointer argument", what);
  JSCC_REQUIRE(!eff || (row_id && ld_eff >= n_vox), "%s: efficiency rows need row ids, ld >= V", what);
  JSCC_REQUIRE(ldx >= n_vox && ldw >= n_vox, "%s: ldx / ldw < n_vox", what);
  JSCC_REQUIRE(n_chunks <= 65535, "%s: %lld chunks exceed the grid's y extent", what, (long long)n_chunks);
  const size_t need = jscc_compton_batch_workspace_bytes(n_ev, n_chunks, n_vox);
  JSCC_REQUIRE(workspace && workspace_bytes >= need, "%s: workspace too small (%zu < %zu)", what, workspace_bytes,
               need);
  Carver cv(workspace, workspace_bytes);
  const int64_t ldp = (int64_t)align_up((size_t)n_vox, 8);
  float* f = cv.take<float>((size_t)n_ev);
  float* q = cv.take<float>((size_t)n_ev);
  float* part = cv.take<float>((size_t)n_chunks * ldp);
  JSCC_REQUIRE(cv.ok(), "%s: workspace carve overflow", what);
  cudaStream_t st = as_stream(stream);
  const ConeEvent* rec = reinterpret_cast<const ConeEvent*>(records);
  const unsigned fgrid = (unsigned)(n_ev / 16);
  dim3 bgrid((unsigned)((n_vox + kConeThreads - 1) / kConeThreads), (unsigned)n_chunks);
  int64_t rb = (n_ev + 255) / 256;
  if (rb > 4096) rb = 4096;
  if (eff_dtype == JSCC_DTYPE_F32) {
    const float* e = static_cast<const float*>(eff);
    JSCC_TIMED("cone_forward", st,
               (cone_forward_pair_kernel<false, float, true><<<fgrid, kConeThreads, 0, st>>>(
                   rec, row_id, n_ev, coor, n_vox, X, e, ld_eff, f, block_inst, ldx, n_inst)));
    JSCC_LAUNCH_CHECK();
    JSCC_TIMED("cone_ratio", st,
               (cone_ratio_batch_kernel<<<(unsigned)rb, 256, 0, st>>>(f, event_inst, n_ev, n_inst, q)));
    JSCC_LAUNCH_CHECK();
    JSCC_TIMED("cone_back", st,
               (cone_back_pair_kernel<false, float, true><<<bgrid, kConeThreads, 0, st>>>(
                   rec, row_id, n_ev, 0, q, coor, n_vox, e, ld_eff, part, ldp, chunk_range)));
  } else {
    const __nv_bfloat16* e = static_cast<const __nv_bfloat16*>(eff);
    JSCC_TIMED("cone_forward", st,
               (cone_forward_pair_kernel<false, __nv_bfloat16, true><<<fgrid, kConeThreads, 0, st>>>(
                   rec, row_id, n_ev, coor, n_vox, X, e, ld_eff, f, block_inst, ldx, n_inst)));
    JSCC_LAUNCH_CHECK();
    JSCC_TIMED("cone_ratio", st,
               (cone_ratio_batch_kernel<<<(unsigned)rb, 256, 0, st>>>(f, event_inst, n_ev, n_inst, q)));
    JSCC_LAUNCH_CHECK();
    JSCC_TIMED("cone_back", st,
               (cone_back_pair_kernel<false, __nv_bfloat16, true><<<bgrid, kConeThreads, 0, st>>>(
                   rec, row_id, n_ev, 0, q, coor, n_vox, e, ld_eff, part, ldp, chunk_range)));
  }
  JSCC_LAUNCH_CHECK();
  int64_t blocks = ((int64_t)n_inst * n_vox + 255) / 256;
  if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
  JSCC_TIMED("cone_batch_reduce", st,
             (cone_batch_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(part, ldp, n_chunks, inst_chunk, n_inst,
                                                                          n_vox, scale != 1.0f ? 1 : 0, scale, W,
                                                                          ldw)));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_compton_project(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor, int64_t n_vox,
                         int32_t model, int32_t use_window, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                         const float* img, const int64_t* rotmat, int64_t ld_rot, float* f_out, void* workspace,
                         size_t workspace_bytes, void* stream) {
  return compton_stage_entry("jscc_compton_project", 1, records, row_id, n_ev, coor, n_vox, model, use_window, eff,
                             eff_dtype, ld_eff, img, rotmat, nullptr, ld_rot, nullptr, f_out, 1.f, nullptr, workspace,
                             workspace_bytes, stream);
}

int jscc_compton_backproject(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor,
                             int64_t n_vox, int32_t model, int32_t use_window, const void* eff, int32_t eff_dtype,
                             int64_t ld_eff, const float* g, const int64_t* rotmat_inv, int64_t ld_rot, float scale,
                             float* weight, void* workspace, size_t workspace_bytes, void* stream) {
  return compton_stage_entry("jscc_compton_backproject", 2, records, row_id, n_ev, coor, n_vox, model, use_window, eff,
                             eff_dtype, ld_eff, nullptr, nullptr, rotmat_inv, ld_rot, g, nullptr, scale, weight,
                             workspace, workspace_bytes, stream);
}

static int compton_f64_entry(const char* what, int stage, const float* records, const int32_t* row_id, int64_t n_ev,
                             const float* coor, int64_t n_vox, int32_t model, const void* eff, int32_t eff_dtype,
                             int64_t ld_eff, const double* in, double scale, double* out, void* stream) {
  JSCC_REQUIRE(n_ev >= 0 && n_vox >= 0, "%s: negative size", what);
  JSCC_REQUIRE(model == JSCC_CONE_STRICT, "%s: the FP64 evaluation implements the strict model only", what);
  JSCC_REQUIRE(eff_dtype == JSCC_DTYPE_F32 || eff_dtype == JSCC_DTYPE_BF16, "%s: bad dtype", what);
  if (n_ev == 0 || n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(records && coor && in && out, "%s: null pointer argument", what);
  JSCC_REQUIRE(!eff || (row_id && ld_eff >= n_vox), "%s: efficiency rows need row ids, ld >= V", what);
  cudaStream_t st = as_stream(stream);
  const ConeEvent* rec = reinterpret_cast<const ConeEvent*>(records);
  const int64_t cap = (int64_t)num_sms() * 8;
  if (stage == 1) {
    const unsigned grid = (unsigned)(n_ev < cap ? n_ev : cap);
    if (eff_dtype == JSCC_DTYPE_BF16)
      JSCC_TIMED("cone_forward_f64", st,
                 (cone_forward_f64_kernel<__nv_bfloat16><<<grid, 256, 0, st>>>(
                     rec, row_id, n_ev, coor, n_vox, in, static_cast<const __nv_bfloat16*>(eff), ld_eff, out)));
    else
      JSCC_TIMED("cone_forward_f64", st,
                 (cone_forward_f64_kernel<float><<<grid, 256, 0, st>>>(rec, row_id, n_ev, coor, n_vox, in,
                                                                      static_cast<const float*>(eff), ld_eff, out)));
  } else {
    int64_t blocks = (n_vox + 255) / 256;
    if (blocks > cap) blocks = cap;
    if (eff_dtype == JSCC_DTYPE_BF16)
      JSCC_TIMED("cone_back_f64", st,
                 (cone_back_f64_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, st>>>(
                     rec, row_id, n_ev, coor, n_vox, in, static_cast<const __nv_bfloat16*>(eff), ld_eff, scale, out)));
    else
      JSCC_TIMED("cone_back_f64", st,
                 (cone_back_f64_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
                     rec, row_id, n_ev, coor, n_vox, in, static_cast<const float*>(eff), ld_eff, scale, out)));
  }
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}

int jscc_compton_project_f64(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor,
                             int64_t n_vox, int32_t model, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                             const double* img, double* f_out, void* stream) {
  return compton_f64_entry("jscc_compton_project_f64", 1, records, row_id, n_ev, coor, n_vox, model, eff, eff_dtype,
                           ld_eff, img, 1.0, f_out, stream);
}

int jscc_compton_backproject_f64(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor,
                                 int64_t n_vox, int32_t model, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                                 const double* g, double scale, double* weight, void* stream) {
  return compton_f64_entry("jscc_compton_backproject_f64", 2, records, row_id, n_ev, coor, n_vox, model, eff,
                           eff_dtype, ld_eff, g, scale, weight, stream);
}

int jscc_take_bad_detector_count(unsigned int* out) {
  unsigned int h = 0, zero = 0;
  JSCC_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_bad_detector_count, sizeof(h)));
  JSCC_CUDA_CHECK(cudaMemcpyToSymbol(g_bad_detector_count, &zero, sizeof(zero)));
  if (out) *out = h;
  return JSCC_OK;
}

}  // extern "C"
