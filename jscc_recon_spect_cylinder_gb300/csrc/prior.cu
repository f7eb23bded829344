// Relative-difference prior (Nuyts et al., IEEE Trans. Nucl. Sci. 49(1):56-60, 2002) over a
// symmetric neighbour table, value and gradient in one pass:
//
//   R(x)      = 1/2 sum_j sum_{k in N(j)} w_jk phi(x_j, x_k)
//   phi(a, b) = d^2 / D,   d = a - b,   D = a + b + gamma |d| + eps
//   dR/dx_j   = sum_{k in N(j)} w_jk dphi/da(x_j, x_k)
//   dphi/da   = d (2 D - d (1 + gamma sgn d)) / D^2 = d (a + 3 b + gamma |d| + 2 eps) / D^2
//
// phi is symmetric in (a, b) and the table holds every edge in both directions with the same
// weight, so the gradient is a gather over the voxel's own neighbours (no atomics). The value
// is reduced in a fixed order: each block writes its sum (warp shuffles, then warps in order)
// to a caller workspace slot, and a one-block second pass adds the slots in order, so the
// value is bit-identical from call to call. The table
// is neighbour-major ([K, V]: nbr[k * V + j]) so a warp's loads of one neighbour slot are
// coalesced; slot entries of -1 are padding. The image is only gathered from (36,000 voxels
// at the 100 x 360 grid: 144 KB, L1/L2 resident), so the pass streams the 8 bytes per slot
// of the table and writes 4 bytes per voxel.
#include "jscc_common.cuh"

namespace jscc {

constexpr int kPriorThreads = 256;

__device__ unsigned int g_prior_bad_index_count = 0;  // out-of-range neighbour indices seen

// Read and clear this unit's counter (jscc_take_bad_index_count adds it to its own).
unsigned int take_prior_bad_index_count() {
  unsigned int h = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&h, g_prior_bad_index_count, sizeof(h)) != cudaSuccess) return 0;
  cudaMemcpyToSymbol(g_prior_bad_index_count, &zero, sizeof(zero));
  return h;
}

template <typename R>
__global__ void __launch_bounds__(kPriorThreads)
rdp_prior_kernel(const R* __restrict__ x, const int32_t* __restrict__ nbr, const float* __restrict__ wt,
                 int64_t n_vox, int n_nbr, R gamma, R eps, R beta, double* __restrict__ block_sums,
                 R* __restrict__ grad, int accumulate) {
  __shared__ R red[kPriorThreads / 32];
  R part = 0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_vox;
       j += (int64_t)gridDim.x * blockDim.x) {
    const R a = x[j];
    R g = 0;
    for (int k = 0; k < n_nbr; ++k) {
      const int32_t i = nbr[(int64_t)k * n_vox + j];
      if (i < 0) continue;
      if ((int64_t)i >= n_vox) {  // corrupt table: counted for the host, access skipped
        atomicAdd(&g_prior_bad_index_count, 1u);
        continue;
      }
      const R b = x[i];
      const R w = (R)wt[(int64_t)k * n_vox + j];
      const R d = a - b;
      if (d == (R)0) continue;  // phi and its derivative vanish (and D may be 0)
      const R ad = fabs(d);
      const R D = a + b + gamma * ad + eps;
      const R inv = (R)1 / D;
      part += w * d * d * inv;
      g += w * d * (a + (R)3 * b + gamma * ad + (R)2 * eps) * inv * inv;
    }
    if (grad != nullptr) grad[j] = (accumulate ? grad[j] : (R)0) + beta * g;
  }
  if (block_sums == nullptr) return;
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0.0;
    for (int w = 0; w < kPriorThreads / 32; ++w) acc += (double)red[w];
    block_sums[blockIdx.x] = acc;
  }
}

// *value += beta / 2 * sum_b block_sums[b]: each thread adds a strided run of the slots in
// order, then the threads' sums are added in thread order (one block, fixed order).
__global__ void __launch_bounds__(kPriorThreads)
rdp_value_kernel(const double* __restrict__ block_sums, int n_blocks, double half_beta, double* __restrict__ value) {
  __shared__ double red[kPriorThreads];
  double acc = 0.0;
  for (int b = threadIdx.x; b < n_blocks; b += kPriorThreads) acc += block_sums[b];
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kPriorThreads; ++i) t += red[i];
    *value += half_beta * t;
  }
}

static int64_t rdp_blocks(int64_t n_vox) {
  int64_t blocks = (n_vox + kPriorThreads - 1) / kPriorThreads;
  const int64_t cap = (int64_t)num_sms() * 8;
  return blocks > cap ? cap : blocks;
}

}  // namespace jscc

using namespace jscc;

extern "C" size_t jscc_rdp_prior_workspace_bytes(int64_t n_vox) {
  return n_vox <= 0 ? 0 : (size_t)rdp_blocks(n_vox) * sizeof(double);
}

template <typename R>
static int rdp_entry(const R* img, const int32_t* nbr, const float* weight, int64_t n_vox, int32_t n_nbr, R gamma,
                     R eps, R beta, double* value, R* grad, int32_t accumulate, void* workspace,
                     size_t workspace_bytes, void* stream) {
  JSCC_REQUIRE(n_vox >= 0 && n_vox <= INT32_MAX, "jscc_rdp_prior: n_vox %lld out of range", (long long)n_vox);
  JSCC_REQUIRE(n_nbr >= 0 && n_nbr <= 64, "jscc_rdp_prior: n_nbr %d out of range [0, 64]", n_nbr);
  JSCC_REQUIRE(gamma >= 0 && eps >= 0, "jscc_rdp_prior: gamma and eps must be >= 0");
  JSCC_REQUIRE(value != nullptr || grad != nullptr, "jscc_rdp_prior: neither value nor grad requested");
  if (n_vox == 0) return JSCC_OK;
  JSCC_REQUIRE(img != nullptr && (n_nbr == 0 || (nbr != nullptr && weight != nullptr)),
               "jscc_rdp_prior: null pointer argument");
  const int64_t blocks = rdp_blocks(n_vox);
  double* block_sums = nullptr;
  if (value != nullptr) {
    JSCC_REQUIRE(workspace != nullptr && workspace_bytes >= (size_t)blocks * sizeof(double),
                 "jscc_rdp_prior: workspace of %zu bytes is smaller than the %zu bytes needed", workspace_bytes,
                 (size_t)blocks * sizeof(double));
    JSCC_REQUIRE(reinterpret_cast<uintptr_t>(workspace) % 8 == 0, "jscc_rdp_prior: workspace not 8-byte aligned");
    block_sums = static_cast<double*>(workspace);
  }
  cudaStream_t st = as_stream(stream);
  JSCC_TIMED("rdp_prior", st,
             rdp_prior_kernel<R><<<(unsigned)blocks, kPriorThreads, 0, st>>>(img, nbr, weight, n_vox, n_nbr, gamma,
                                                                           eps, beta, block_sums, grad, accumulate));
  JSCC_LAUNCH_CHECK();
  if (value != nullptr) {
    JSCC_TIMED("rdp_value", st,
               rdp_value_kernel<<<1, kPriorThreads, 0, st>>>(block_sums, (int)blocks, 0.5 * (double)beta, value));
    JSCC_LAUNCH_CHECK();
  }
  return JSCC_OK;
}

extern "C" int jscc_rdp_prior(const float* img, const int32_t* nbr, const float* weight, int64_t n_vox,
                              int32_t n_nbr, float gamma, float eps, float beta, double* value, float* grad,
                              int32_t accumulate, void* workspace, size_t workspace_bytes, void* stream) {
  return rdp_entry<float>(img, nbr, weight, n_vox, n_nbr, gamma, eps, beta, value, grad, accumulate, workspace,
                          workspace_bytes, stream);
}

extern "C" int jscc_rdp_prior_f64(const double* img, const int32_t* nbr, const float* weight, int64_t n_vox,
                                  int32_t n_nbr, double gamma, double eps, double beta, double* value, double* grad,
                                  int32_t accumulate, void* workspace, size_t workspace_bytes, void* stream) {
  return rdp_entry<double>(img, nbr, weight, n_vox, n_nbr, gamma, eps, beta, value, grad, accumulate, workspace,
                           workspace_bytes, stream);
}
