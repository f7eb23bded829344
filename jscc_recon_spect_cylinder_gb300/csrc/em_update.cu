// EM image update: x <- x * w / s in the reference's two flavours.
//
// Plain (recon_osem_plane.py:54, :73, :118):    x * w / s with w = (2-a) w_c + a w_s in joint mode.
// Safe  (recon_osem_plane_sparse.py:60-66):     nan/inf -> 0 in w and s; where s > eps,
//                                                x * max(w, 0) / s, else 0.
// Every product and sum is rounded separately (no FMA contraction) so the update
// rounds exactly like the reference's sequence of elementwise tensor ops.
#include "jscc_common.cuh"

namespace jscc {

__device__ __forceinline__ float finite_or_zero(float v) { return isfinite(v) ? v : 0.f; }

__global__ void em_update_kernel(float* __restrict__ out, const float* __restrict__ img,
                                 const float* __restrict__ wa, int has_ca, float ca,
                                 const float* __restrict__ wb, float cb,
                                 const float* __restrict__ s, int64_t n, int mode, float eps) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    float w = wa[j];
    if (has_ca) w = __fmul_rn(ca, w);
    if (wb != nullptr) w = __fadd_rn(w, __fmul_rn(cb, wb[j]));
    const float x = img[j];
    float sj = s[j];
    float r;
    if (mode == JSCC_EM_PLAIN) {
      r = __fdiv_rn(__fmul_rn(x, w), sj);
    } else {
      w = finite_or_zero(w);
      sj = finite_or_zero(sj);
      r = (sj > eps) ? __fdiv_rn(__fmul_rn(x, fmaxf(w, 0.f)), sj) : 0.f;
    }
    out[j] = r;
  }
}

}  // namespace jscc

using namespace jscc;

extern "C" int jscc_em_update(float* img_out, const float* img, const float* w_a,
                              int32_t has_coef_a, float coef_a, const float* w_b, float coef_b,
                              const float* s_map, int64_t n_vox, int32_t mode, float eps,
                              void* stream) {
  JSCC_REQUIRE(n_vox >= 0, "jscc_em_update: negative n_vox");
  JSCC_REQUIRE(mode == JSCC_EM_PLAIN || mode == JSCC_EM_SAFE, "jscc_em_update: bad mode %d", mode);
  if (n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(img_out && img && w_a && s_map, "jscc_em_update: null pointer argument");
  int64_t blocks = (n_vox + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 16;
  if (blocks > cap) blocks = cap;
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("em_update", st,
             em_update_kernel<<<(unsigned)blocks, 256, 0, st>>>(img_out, img, w_a, has_coef_a, coef_a,
                                                                w_b, coef_b, s_map, n_vox, mode, eps));
  JSCC_LAUNCH_CHECK();
  return JSCC_OK;
}
