/*
 * jscc_gb300.h — C-ABI of the GB300 (sm_103a) OSEM hot path for SC / JSCC
 * (self-collimation + joint Compton) SPECT reconstruction on a polar grid.
 *
 * Conventions shared by every entry point
 *  - Plain device pointers and sizes; no framework types cross this boundary.
 *  - Images are dense float32 vectors of n_vox voxels (the reference's [V, 1]).
 *  - Matrices are row-major with an explicit leading dimension (elements).
 *  - Rotation tables keep the reference layout: int64, 1-based, shape
 *    [n_vox, n_rot] row-major (column r is the reference's rotmat[:, r]).
 *  - `stream` is a cudaStream_t passed as void*; all work is enqueued on it
 *    and every entry point returns without synchronising.
 *  - No entry point allocates device memory. Temporary buffers come from a
 *    caller-provided workspace whose size the matching *_workspace_bytes()
 *    function returns for the same problem sizes.
 *  - Return value: JSCC_OK, or an error code with a message available from
 *    jscc_last_error() (thread-local).
 *  - Results are deterministic: reductions run in a fixed order and no float
 *    atomics are used, so repeated calls give bit-identical outputs.
 */
#ifndef JSCC_GB300_H
#define JSCC_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define JSCC_API __attribute__((visibility("default")))
#else
#define JSCC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define JSCC_OK 0
#define JSCC_ERR_INVALID 1 /* bad argument (shape, size, alignment, null) */
#define JSCC_ERR_CUDA 2    /* a CUDA runtime call or launch failed */

#define JSCC_DTYPE_F32 0
#define JSCC_DTYPE_BF16 1

/* ---------------------------------------------------------------- runtime */

/* Message of the last error raised on the calling thread ("" if none). */
JSCC_API const char* jscc_last_error(void);

/* ABI version of this library; bumped whenever a signature changes. */
JSCC_API int jscc_abi_version(void);

/* Number of kernels this library has launched since load / last reset. */
JSCC_API unsigned long long jscc_launch_count(void);
JSCC_API void jscc_reset_launch_count(void);

/*
 * Kernels never read or write out of bounds on a bad 1-based rotation index
 * (the reference's index_select raises for those, recon_osem_plane.py:51); they
 * skip the element and count it. This returns the count since the last call
 * and resets it (synchronous device read).
 */
JSCC_API int jscc_take_bad_index_count(unsigned int* out);

/*
 * Per-kernel timing for measurement runs: while enabled, every kernel launch is
 * bracketed by CUDA events on its own stream. collect() waits for the recorded
 * events and writes one line per kernel, "name launches total_ms\n", into buf
 * (truncated to buf_bytes), then clears the record. Do not enable it while a
 * stream is being captured into a CUDA graph.
 */
JSCC_API void jscc_kernel_timing_enable(int enable);
JSCC_API int jscc_kernel_timing_collect(char* buf, size_t buf_bytes);

/* ------------------------------------------------ single-photon (SC) path */

/*
 * Workspace bytes needed by jscc_sc_weight for the given sizes.
 */
JSCC_API size_t jscc_sc_weight_workspace_bytes(int64_t n_bins, int64_t n_vox, int32_t n_rot);

/*
 * SC weight of one subset block, accumulated over all rotations:
 *
 *   for r in 0..n_rot-1:
 *     x_r[j]  = img[rotmat[j * ld_rot + r] - 1]      (identity if rotmat == NULL)
 *     f[b]    = sum_j A[rb, j] * x_r[j]              (rb = row_idx ? row_idx[b] : b)
 *     q[b]    = proj[rb, r] / (use_floor ? max(f[b], floor) : f[b])
 *     u[j]    = sum_b A[rb, j] * q[b]
 *     weight[j] += scale * u[rotmat_inv[j * ld_rot + r] - 1]  (identity if NULL)
 *
 * Replaces, per call, the inner rotation loop of
 *   recon_osem_plane.py:49-53 (osem_bin_mode; get_weight_single :28-30, use_floor = 0),
 *   recon_osem_local_cntstat.py:215-222 (osem_bin_mode_local; clamped get_weight_single :6-8),
 *   recon_osem_local_sparse_jsccsd_only.py:356-360 (joint local, scale = alpha),
 *   recon_osem_plane_sparse.py:96-100 (osem_joint_mode_sparse, SC half).
 * A single rotation with NULL tables is recon_osem_plane.py:28-30 itself.
 *
 * A:      rows of lda elements, dtype a_dtype (JSCC_DTYPE_F32 or JSCC_DTYPE_BF16)
 * row_idx: optional [n_bins] int64 0-based row ids into A and proj (a subset
 *         selected without copying A, recon_osem_local_cntstat.py:11-25); NULL
 *         means rows 0..n_bins-1. Ids must be in range: they are not checked.
 * proj:   [n_bins, ld_proj] float32, column r used for rotation r
 * weight: [n_vox] float32, accumulated in place (caller zeroes it first)
 * rotmat, rotmat_inv: int64 1-based tables with row stride ld_rot (elements);
 *         pointing at column c of a [V, R] table with ld_rot = R selects
 *         rotations c..c+n_rot-1.
 */
JSCC_API int jscc_sc_weight(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox,
                   const float* proj, int64_t ld_proj, int32_t n_rot, const float* img,
                   const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot,
                   int32_t use_floor, float floor, float scale, float* weight, void* workspace,
                   size_t workspace_bytes, void* stream);

/*
 * jscc_sc_weight without a workspace: the same computation and arguments minus
 * (workspace, workspace_bytes). No counterpart in the reference (its PyTorch code
 * allocates freely); it exists for callers that cannot allocate device memory — a
 * host framework that owns all GPU memory through its own pool and forbids
 * allocations from plugins, a runtime reaching this library over a bare FFI with
 * no device allocator, or a latency-critical loop that must avoid cudaMalloc's
 * implicit synchronisation.
 *
 * Scratch lives in one fixed device array of JSCC_SC_NOALLOC_SCRATCH_BYTES (16 MiB)
 * inside this library; every GPU that loads the library holds it until the process
 * exits. Problems whose scratch need (jscc_sc_weight_workspace_bytes) exceeds it are
 * rejected with JSCC_ERR_INVALID and a message; use jscc_sc_weight for those. The
 * 16 MiB covers e.g. a 10,240-bin x 36,000-voxel subset block with one rotation
 * (about 5 MiB); scratch grows with the rotations handled per pass (up to 8).
 * The first call on each device looks up the array's device address (with that
 * device current); make that first call before any stream capture. All calls share
 * the one array, so calls that can overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. Nothing in the scratch needs
 * clearing between calls: each call writes every scratch byte it later reads.
 * Calls no cudaMalloc / cudaFree and no allocating library routine.
 */
#define JSCC_SC_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
JSCC_API int jscc_sc_weight_noalloc(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, const float* proj, int64_t ld_proj,
                   int32_t n_rot, const float* img, const int64_t* rotmat,
                   const int64_t* rotmat_inv, int64_t ld_rot, int32_t use_floor, float floor,
                   float scale, float* weight, void* stream);

/* ------------------------------------------------------------ EM update */

#define JSCC_EM_PLAIN 0 /* img * w / s                         (recon_osem_plane.py:54, :73, :118) */
#define JSCC_EM_SAFE 1  /* safe_em_update                      (recon_osem_plane_sparse.py:60-66) */

/*
 * img_out[j] = EM(img[j], w[j], s_map[j]) with
 *   w = coef_a * w_a + coef_b * w_b   (w_b may be NULL; coef multiplies are
 *                                      skipped when has_coef_a == 0, matching
 *                                      the reference's un-scaled weight)
 * JSCC_EM_PLAIN: (img * w) / s.
 * JSCC_EM_SAFE:  nan/inf -> 0 in w and s; s > eps ? img * max(w, 0) / s : 0.
 * Replaces recon_osem_plane.py:54, :73, :117-118 and recon_osem_plane_sparse.py:60-66, :110-111.
 * img_out may alias img.
 */
JSCC_API int jscc_em_update(float* img_out, const float* img, const float* w_a, int32_t has_coef_a,
                   float coef_a, const float* w_b, float coef_b, const float* s_map, int64_t n_vox,
                   int32_t mode, float eps, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JSCC_GB300_H */
