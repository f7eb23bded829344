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
 *  - Per-device state is cached for the life of the process (kernel attributes set
 *    once per device, the no-allocation scratch address): after cudaDeviceReset on a
 *    device, do not use the library on that device again in the same process.
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
/* Adds n to the launch count: the kernels of this library that one replay of a captured
 * CUDA graph launches (the replay itself does not pass through the library). */
JSCC_API void jscc_count_graph_launches(unsigned long long n);

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
 * Workspace bytes for jscc_sc_weight at the given sizes: the two-pass kernels' scratch
 * (forward split, ratio, back-projection partials: the minimum jscc_sc_weight accepts)
 * plus, for one rotation, one partial image per cluster of the fused single-read kernel,
 * which jscc_sc_weight runs instead of the two passes when the workspace holds them (the
 * image read directly, no rotation tables, 16-byte-aligned rows, at most 38,400 voxels).
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
 * The two halves of jscc_sc_weight on their own — the forward and the adjoint of the SC
 * projector, for a differentiable projector (no counterpart in the reference, whose autograd
 * would go through torch.matmul; its backprojection is the transpose used in
 * recon_osem_plane.py:28-30):
 *
 *   jscc_sc_project:     out[b * ld_out + r] = sum_j A[rb, j] * img[rotmat[j * ld_rot + r] - 1]
 *   jscc_sc_backproject: weight[j] += scale * sum_r u_r[rotmat_inv[j * ld_rot + r] - 1],
 *                        u_r = A^T g[:, r]   (g [n_bins, ld_g], column r)
 *
 * for r < n_rot (rotation tables NULL: identity, n_rot = 1). Workspace:
 * jscc_sc_weight_workspace_bytes(n_bins, n_vox, n_rot). Same kernels and reduction orders as
 * jscc_sc_weight.
 */
JSCC_API int jscc_sc_project(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, int32_t n_rot, const float* img,
                   const int64_t* rotmat, int64_t ld_rot, float* out, int64_t ld_out,
                   void* workspace, size_t workspace_bytes, void* stream);
JSCC_API int jscc_sc_backproject(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, int32_t n_rot, const float* g, int64_t ld_g,
                   const int64_t* rotmat_inv, int64_t ld_rot, float scale, float* weight,
                   void* workspace, size_t workspace_bytes, void* stream);

/*
 * SC sensitivity (column sums of the system matrix through the inverse rotations):
 *
 *   weight[j] += (sum_{r < n_rot} colsum(A)[rotmat_inv[j * ld_rot + r] - 1]) / n_rot,
 *   colsum(A)[c] = sum_b A[rb, c]   (rb = row_idx ? row_idx[b] : b)
 *
 * Replaces main_local_cntstat.py:140-146 (compute_sensitivity_local) and the s_map_s loop of
 * main_plane_sparse.py:440-444 (one call per energy; the caller sums energies). rotmat_inv
 * NULL means the identity (n_rot must then be 1). Workspace:
 * jscc_sc_weight_workspace_bytes(n_bins, n_vox, 1). The sum over rows is Kahan-compensated
 * (within row chunks, then over the chunk sums and their carried errors, in a fixed order:
 * deterministic, and within a few ulp of the exact column sum for any row count).
 */
JSCC_API int jscc_sc_sensitivity(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, int32_t n_rot, const int64_t* rotmat_inv,
                   int64_t ld_rot, float* weight, void* workspace, size_t workspace_bytes,
                   void* stream);

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
 * exits. Problems whose two-pass scratch need exceeds it are rejected with
 * JSCC_ERR_INVALID and a message; use jscc_sc_weight for those. The 16 MiB covers e.g. a
 * 10,240-bin x 36,000-voxel subset block with one rotation (about 5 MiB for the two
 * passes); scratch grows with the rotations handled per pass (up to 8). The fused
 * single-read kernel runs when the scratch also holds its partial images (see
 * jscc_sc_weight_workspace_bytes).
 * The first call on each device looks up the array's device address (with that
 * device current); make that first call before any stream capture. The address is
 * kept for the life of the process: after cudaDeviceReset on a device, do not call this
 * entry point on that device again in the same process (the array may then live at
 * another address). All calls share
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

/* ------------------------------------------------------- Compton cone (kernel a) */

#define JSCC_CONE_STRICT 0 /* process_list_plane_strict.py (kinematic filter, clamped angles) */
#define JSCC_CONE_LEGACY 1 /* process_list_plane.py (derivative sigma_E, atan sigma_pos, no clamps) */
#define JSCC_CONE_SIMPLE 2 /* exp(-(beta - theta)^2 / (2 sigma_E^2)) / d01^2 on strict records (no sigma_pos,
                              no Klein-Nishina factor): the simplified list-mode kernel */
#define JSCC_CONE_RECORD_FLOATS 16 /* floats per event record (64 bytes, 16-byte aligned) */

/*
 * Event selection and per-event record of the Compton cone kernel, for a list that
 * is already energy-smeared (the caller smears with the reference's torch.randn draws).
 * Keeps event i when, with float32 arithmetic in the reference's operation order,
 *   e1 < thr_max, e1 > thr_min, e2 > thr_min, e1 + e2 > thr_sum
 *   (strict only) -1 + 1e-6 < 1 - 0.511 e1 / ((e0 - e1) e0) < 1 - 1e-6
 *   |y(cp1) - y(cp2)| > 0.1
 * (process_list_plane_strict.py:164-189, :30-36; process_list_plane.py:30-46). For kept
 * events it writes the 16-float record (first-hit position, pos2 - pos1, |pos2 - pos1|,
 * Compton angle (FP64 when theta_fp64), sigma_E branches (:39-52), Klein-Nishina factor,
 * per-axis sigma1^2 + sigma2^2 from the given tables (:59-96), and a cos(beta) window of
 * +-window_sigmas bounding sigmas; window_sigmas <= 0 disables pruning) and
 * row_id = cp1 - 1. Detector ids outside [1, n_det] drop the event and are counted
 * (jscc_take_bad_detector_count).
 * list: [n_events, ld_list] float32 rows (cp1, e1, cp2, e2); det_pos [n_det, 3];
 * sig1_sq / sig2_sq [n_det, 3] (strict) ; keep [n_events] uint8; records 16-byte aligned.
 */
JSCC_API int jscc_compton_event_prep(const float* list, int64_t ld_list, int64_t n_events,
                   const float* det_pos, const float* sig1_sq, const float* sig2_sq,
                   int64_t n_det, float e0, float ene_resolution, float thr_max,
                   float thr_min, float thr_sum, int32_t model, int32_t theta_fp64,
                   float window_sigmas, float delta_r1, float delta_r2, uint8_t* keep,
                   float* records, int32_t* row_id, void* stream);

/*
 * Materialised cone rows for the T builders (process_list_plane_strict.py:201-240,
 * process_list_plane.py:56-95, process_list_plane_sparse.py:78-106):
 *   t_compton[i, j] = cone(record i, coor j)            (every pair, no window)
 *   t[i, j]         = t_compton[i, j] * eff[row_id[i], j]  (eff may be NULL: t = t_compton)
 * coor [V, 3] float32; eff rows of ld_eff elements (float32 or bf16); either output may
 * be NULL. At most 65,535 events per call.
 */
JSCC_API int jscc_compton_cone_rows(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t V, int32_t model, const void* eff,
                   int32_t eff_dtype, int64_t ld_eff, float* t_compton, float* t,
                   void* stream);

/*
 * Per-event row statistics of t = cone * eff without storing the row: s1 = sum_j t,
 * s2 = sum_j t^2, nan_flag = any NaN. Feeds the NaN/zero-row filter and the
 * effective-support filter (process_list_plane_strict.py:137-148, :241-246) of the
 * fused path. use_window applies the record's cos(beta) window (strict model only).
 */
JSCC_API int jscc_compton_row_stats(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t V, int32_t model, int32_t use_window,
                   const void* eff, int32_t eff_dtype, int64_t ld_eff, float* s1, float* s2,
                   int32_t* nan_flag, void* stream);

JSCC_API size_t jscc_compton_weight_workspace_bytes(int64_t n_ev, int64_t n_vox);

/*
 * Fused list-mode Compton weight with T recomputed on the fly (never stored):
 *   x_r = img[rotmat[:, 0] - 1]            (identity when rotmat == NULL)
 *   f_i = sum_j t_ij x_r[j],  t_ij = cone(record i, coor j) * eff[row_id[i], j]
 *   u_j = sum_i t_ij / f_i
 *   weight[j] += scale * u[rotmat_inv[j * ld_rot] - 1]
 * Replaces get_weight_compton (recon_osem_plane.py:33-42) over the rows of the strict or
 * legacy builder, inside osem_list_mode / osem_joint_mode (:63-125): the builder's row
 * normalisation does not change the weight. Events must already be filtered (event_prep
 * + row_stats). use_window prunes pairs outside the record's window (t < exp(-K^2/2)).
 */
JSCC_API int jscc_compton_weight(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t n_vox, int32_t model, int32_t use_window,
                   const void* eff, int32_t eff_dtype, int64_t ld_eff, const float* img,
                   const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, float scale,
                   float* weight, void* workspace, size_t workspace_bytes, void* stream);

/* Detector ids outside the table seen by jscc_compton_event_prep since the last call
 * (synchronous device read; resets the count). */
JSCC_API int jscc_take_bad_detector_count(unsigned int* out);

/*
 * jscc_compton_weight (strict model, every pair) for several instances in one launch per
 * direction: instance b's events reweight its own image, W[b] += scale * T_b^T (1 / T_b X[b])
 * (recon_osem_plane.py:33-42 per instance, as the joint loops use it, with T recomputed on the
 * fly). The events of all instances are concatenated; the device tables describe the segments:
 *   event_inst  [n_ev]          instance of each event, -1 for padding events (no contribution)
 *   block_inst  [n_ev / 16]     instance of each 16-event forward block (each block holds events of
 *                               one instance and padding only; pad every instance to a multiple of 16)
 *   chunk_range [n_chunks + 1]  event offsets of the back-projection chunks (a chunk holds events
 *                               of one instance only)
 *   inst_chunk  [n_inst + 1]    chunk offsets of each instance (its chunks are consecutive)
 * X [n_inst, ldx] images, W [n_inst, ldw] accumulated (the caller zeroes it). Chunk partial
 * images are summed per instance in chunk order (no float atomics). Out-of-range instance ids
 * in the tables are skipped and counted (jscc_take_bad_detector_count). Workspace:
 * jscc_compton_batch_workspace_bytes(n_ev, n_chunks, n_vox). No counterpart in the reference,
 * which runs one instance at a time: the batched joint reconstruction of many Poisson
 * realisations or count levels.
 */
JSCC_API size_t jscc_compton_batch_workspace_bytes(int64_t n_ev, int64_t n_chunks, int64_t n_vox);
JSCC_API int jscc_compton_weight_batched(const float* records, const int32_t* row_id, int64_t n_ev,
                   const int32_t* event_inst, const int32_t* block_inst, const int64_t* chunk_range,
                   const int32_t* inst_chunk, int64_t n_chunks, int32_t n_inst, const float* coor,
                   int64_t n_vox, const void* eff, int32_t eff_dtype, int64_t ld_eff, const float* X,
                   int64_t ldx, float scale, float* W, int64_t ldw, void* workspace,
                   size_t workspace_bytes, void* stream);

/*
 * The two halves of jscc_compton_weight on their own (T recomputed in both, never stored):
 *   jscc_compton_project:     f_out[i] = sum_j t_ij * rot(img)_j
 *   jscc_compton_backproject: weight[j] += scale * rotinv(sum_i t_ij * g_i)
 * with the same records, row ids, efficiency rows, model and window as jscc_compton_weight
 * (whose workspace size they use). No counterpart in the reference (a differentiable fused
 * projector: the forward and its adjoint).
 */
JSCC_API int jscc_compton_project(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t n_vox, int32_t model, int32_t use_window,
                   const void* eff, int32_t eff_dtype, int64_t ld_eff, const float* img,
                   const int64_t* rotmat, int64_t ld_rot, float* f_out, void* workspace,
                   size_t workspace_bytes, void* stream);
JSCC_API int jscc_compton_backproject(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t n_vox, int32_t model, int32_t use_window,
                   const void* eff, int32_t eff_dtype, int64_t ld_eff, const float* g,
                   const int64_t* rotmat_inv, int64_t ld_rot, float scale, float* weight,
                   void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------ sparse coarse<->fine Compton rows (kernel c) */

/*
 * Separable sparse map of rows, the form of every operator of compton_sparse_ops.py:
 *   out[r][zo * n_lo + lo] = sum_{a in Z[zo]} z_w[a] * sum_{b in L[lo]} l_w[b] * in[rr][z_idx[a] * n_li + l_idx[b]]
 * with rr = row_idx ? row_idx[r] : r and Z, L given as CSR tables (z_ptr [n_zo + 1],
 * l_ptr [n_lo + 1]) built from the reference's dense layer/z matrices:
 *   upsample_coarse_rows_to_fine  (:331-342): L = rows of layer_expand, Z = rows of z_expand
 *   project_fine_rows_to_coarse_adjoint (:345-356): L, Z = columns of layer_expand, z_expand
 *   reduce_fine_rows_to_coarse    (:317-328): L = rows of layer_reduce, Z = rows of z_reduce
 *   reduce_fine_image_to_coarse / upsample_coarse_weight_to_fine (:293-314): one-row forms
 * in: float32 or bf16 rows of ld_in elements; out: float32 rows of ld_out elements.
 * At most 65,535 rows per call.
 */
JSCC_API int jscc_sparse_map(const void* in, int32_t in_dtype, int64_t ld_in, const int32_t* row_idx,
                   int64_t n_rows, float* out, int64_t ld_out, const int32_t* z_ptr,
                   const int32_t* z_idx, const float* z_w, int32_t n_zo, int32_t n_zi,
                   const int32_t* l_ptr, const int32_t* l_idx, const float* l_w, int32_t n_lo,
                   int32_t n_li, void* stream);

/* pack_sparse_event_rows (compton_sparse_ops.py:359-368): rows[i] = (float(cp1[i]), t_compton[i, :]). */
JSCC_API int jscc_sparse_pack(const int64_t* cp1, const float* t_compton, int64_t ld_tc, int64_t n_events,
                   int64_t n_coarse, float* rows, int64_t ld_rows, void* stream);

/* unpack_sparse_event_rows (:371-377), id column: cp1[i] = round-half-even(rows[i, 0]). */
JSCC_API int jscc_sparse_unpack_ids(const float* rows, int64_t ld_rows, int64_t n_events, int64_t* cp1,
                   void* stream);

/*
 * First half of materialize_sparse_event_rows_to_fine (:380-400): for packed rows
 * (cp1, t_compton[V_c]) with upsample taps (two z taps per fine plane: z_taps/z_tw
 * [n_zf, 2]; two layer taps per fine layer: l_taps/l_tw [n_lf, 2]; a missing tap has
 * weight 0), writes fine[i, j] = nan_to_num(up(t_compton_i)[j] * sysmat[clamp(cp1_i - 1), j])
 * and row_sum[i] = sum_j fine[i, j]. The caller keeps rows with a finite positive sum
 * and divides them by it.
 */
JSCC_API int jscc_sparse_materialize(const float* rows, int64_t ld_rows, int64_t n_events,
                   const void* sysmat, int32_t sysmat_dtype, int64_t ld_sysmat, int64_t n_det,
                   const int32_t* z_taps, const float* z_tw, int32_t n_zf, const int32_t* l_taps,
                   const float* l_tw, int32_t n_lf, int32_t n_lc, float* fine, int64_t ld_fine,
                   float* row_sum, void* stream);

#define JSCC_SPARSE_MATERIALIZE 0 /* recon_osem_local_sparse_jsccsd_only.py:13-19 */
#define JSCC_SPARSE_GROUPED 1     /* recon_osem_plane_sparse.py:22-57 */

JSCC_API size_t jscc_sparse_weight_workspace_bytes(int64_t n_events, int64_t n_fine);

/*
 * Fused sparse list-mode weight; fine rows are formed on the fly from the packed coarse
 * rows and never stored:
 *   v_ij = up(t_compton_i)[j] * sysmat[clamp(cp1_i - 1), j]
 *   MATERIALIZE: v = nan_to_num(v); S_i = sum_j v_ij; rows with a non-finite or
 *                non-positive S_i are dropped; c_i = 1 / max((sum_j v_ij x_j) / S_i, 1e-12) / S_i
 *   GROUPED:     c_i = 1 / max(sum_j v_ij x_j, 1e-12)
 *   weight[j] += scale * nan_to_num(sum_i v_ij c_i)   (after the inverse rotation)
 * x is img gathered by rotmat[:, 0] (identity when NULL). Replaces get_weight_compton_sparse
 * in both reference forms and the rotation handling around it (recon_osem_plane_sparse.py:73-80,
 * recon_osem_local_sparse_jsccsd_only.py:362-377).
 */
JSCC_API int jscc_sparse_weight(const float* rows, int64_t ld_rows, int64_t n_events, const void* sysmat,
                   int32_t sysmat_dtype, int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps,
                   const float* z_tw, int32_t n_zf, const int32_t* l_taps, const float* l_tw,
                   int32_t n_lf, int32_t n_lc, int32_t mode, const float* img,
                   const int64_t* rotmat, const int64_t* rotmat_inv, int64_t ld_rot, float scale,
                   float* weight, void* workspace, size_t workspace_bytes, void* stream);

/*
 * jscc_sparse_weight over split storage: row_id [n_events] int32 0-based sysmat rows
 * (cp1 - 1) and t_coarse [n_events, ld_tc] of tc_dtype (float32 or bf16). Same result as
 * jscc_sparse_weight on the packed rows; the split is what lets the coarse rows be stored
 * in BF16 (the packed format keeps cp1 as a float, which BF16 cannot represent).
 */
JSCC_API int jscc_sparse_weight_split(const int32_t* row_id, const void* t_coarse, int32_t tc_dtype,
                   int64_t ld_tc, int64_t n_events, const void* sysmat, int32_t sysmat_dtype,
                   int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps, const float* z_tw,
                   int32_t n_zf, const int32_t* l_taps, const float* l_tw, int32_t n_lf,
                   int32_t n_lc, int32_t mode, const float* img, const int64_t* rotmat,
                   const int64_t* rotmat_inv, int64_t ld_rot, float scale, float* weight,
                   void* workspace, size_t workspace_bytes, void* stream);

/*
 * Grouped form of the sparse weight (same result as jscc_sparse_weight[_split]; the fast
 * path). Events with the same first-hit row g share that sysmat row, so per group
 *   b = adj(A_g * x)                      (adjoint of the upsample, coarse grid)
 *   f_i = t_i . b,  S_i = t_i . adj(A_g)  (per event, coarse grid)
 *   q_g = sum_i c_i t_i                   (per group, coarse grid)
 *   w_j += sum_g A[g, j] * up(q_g)[j]     (fine grid, one thread per voxel)
 * with c_i as in jscc_sparse_weight. Rows come packed (packed_rows, row stride ld_tc) or
 * split (row_id + t_coarse of tc_dtype, stride ld_tc). The host supplies the grouping:
 * order [n_events] (event indices sorted by row), group_offsets [n_groups + 1] into order,
 * group_rows [n_groups] (0-based sysmat rows), and the adjoint as a fixed-width tap table
 * adj_idx / adj_w [adj_width, V_c] (fine index and weight of each tap of coarse voxel c;
 * padding taps have weight 0). event_sums [n_events] holds S_i in MATERIALIZE mode, stored
 * by position in `order` (event_sums[p] = S_order[p]): it is computed when have_sums == 0
 * and only read when have_sums != 0 (S_i depends on the rows, the sysmat and the grouping
 * only, so callers keep it across iterations with the same `order`). The coarse grid must fit in
 * shared memory (V_c floats <= 227 KB). Deterministic (fixed-order reductions).
 * With split rows whose starts are 16-byte aligned and whose pitch (ld_tc) covers the row
 * rounded up to a whole number of 16-byte units (the values past V_c may be anything), and a
 * 16-byte aligned sysmat row pitch, the weight runs as three bulk-copy pipelines: the group
 * adjoints b_g (sysmat row segments streamed into shared memory), the event coefficients and
 * q_g (b_g and the coarse rows streamed in), and the scatter (sysmat tiles and q segments
 * streamed in); their waits are bounded and a wait that gives up is counted
 * (jscc_take_wait_timeout_count), the weight of that call then being invalid.
 * ring_len / ring_stride (0 / 0: no claim) state that the adjoint table is a stride-4 ring
 * stencil: z the identity, each fine plane made of rings of ring_len theta voxels, coarse
 * voxel lc = r * (ring_len / 4) + th with taps r * ring_len + (4 th + d) mod ring_len,
 * d = -3..3, with the polar projector's linear weights 1 - |d| / 4, in each plane (the
 * caller checks the table; the kernels then compute the tap indices, and the weights where
 * they need them, instead of loading them).
 * With BF16 split rows and a BF16 sysmat on one plane of at least four such rings, and the
 * fused cluster kernel enabled (jscc_set_fused_cluster), the per-iteration weight (mode
 * GROUPED, or MATERIALIZE with have_sums) runs as one kernel on clusters of four CTAs that
 * split the rings: each event row and each group's sysmat row is read from HBM once and the
 * per-group coarse sums stay on chip (the per-event sums of MATERIALIZE are computed
 * beforehand by the separate kernels when have_sums == 0).
 */
/*
 * Number of bounded device waits that gave up since the last call (then reset to 0).
 * Nonzero means a bulk copy never completed and the weights computed meanwhile are
 * invalid. No counterpart in the reference (diagnostic of this library's pipeline).
 */
JSCC_API int jscc_take_wait_timeout_count(unsigned int* out);

/*
 * Whether jscc_sparse_weight_grouped uses the fused cluster kernel where it applies
 * (enable != 0) or the separate kernels (adjoints, coefficients, scatter; the default, as they
 * are the faster form on GB300 at the joint configuration's sizes). Process-wide. No
 * counterpart in the reference.
 */
JSCC_API int jscc_set_fused_cluster(int32_t enable);

/*
 * Poll bound of every bounded pipeline wait on the current device: the bulk sparse kernels
 * (jscc_sparse_weight_grouped), the fused single-read SC kernel (jscc_sc_weight,
 * jscc_sc_weight_noalloc) and the tensor-core GEMM (jscc_bf16_gemm_nt). polls < 0
 * restores the default (2^22 polls per wait); 0 makes each such wait give up at once. A CTA
 * that gives up still waits, with a fixed bound of its own, for the copies and MMAs it has
 * in flight, frees its tensor memory and is counted (jscc_take_wait_timeout_count,
 * jscc_take_gemm_timeout_count); the results of that call are invalid. For tests of the
 * give-up path; synchronous. No counterpart in the reference.
 */
JSCC_API int jscc_set_wait_limit(int64_t polls);

JSCC_API size_t jscc_sparse_grouped_workspace_bytes(int64_t n_events, int64_t n_fine, int64_t n_coarse,
                   int32_t n_groups, int32_t adj_width);
JSCC_API int jscc_sparse_weight_grouped(const int32_t* row_id, const void* t_coarse, int32_t tc_dtype,
                   int64_t ld_tc, const float* packed_rows, int64_t n_events, const int32_t* order,
                   const int32_t* group_offsets, const int32_t* group_rows, int32_t n_groups,
                   float* event_sums, int32_t have_sums, const void* sysmat, int32_t sysmat_dtype,
                   int64_t ld_sysmat, int64_t n_det, const int32_t* z_taps, const float* z_tw,
                   int32_t n_zf, const int32_t* l_taps, const float* l_tw, int32_t n_lf, int32_t n_lc,
                   int32_t n_zc, const int32_t* adj_idx, const float* adj_w, int32_t adj_width,
                   int32_t ring_len, int32_t ring_stride,
                   int32_t mode, const float* img, const int64_t* rotmat, const int64_t* rotmat_inv,
                   int64_t ld_rot, float scale, float* weight, void* workspace, size_t workspace_bytes,
                   void* stream);

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

/* ------------------------------------------------ FP64 projector halves and prior */

/*
 * Reference-grade double-precision forms of jscc_sc_project / jscc_sc_backproject,
 * jscc_compton_project / jscc_compton_backproject (strict model, every pair, no rotation
 * tables on the Compton side) and jscc_rdp_prior: the same definitions with double images,
 * projections, adjoint inputs and outputs, every sum in double (the matrix, efficiency rows and
 * event records are read as stored and promoted exactly). For gradient checks of penalised-
 * likelihood objectives against FP64 finite differences; simple kernels, not a hot path.
 * Workspace of jscc_sc_backproject_f64: jscc_sc_f64_workspace_bytes(n_vox, n_rot).
 */
JSCC_API size_t jscc_sc_f64_workspace_bytes(int64_t n_vox, int32_t n_rot);
JSCC_API int jscc_sc_project_f64(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, int32_t n_rot, const double* img, const int64_t* rotmat,
                   int64_t ld_rot, double* out, int64_t ld_out, void* stream);
JSCC_API int jscc_sc_backproject_f64(const void* A, int32_t a_dtype, int64_t lda, const int64_t* row_idx,
                   int64_t n_bins, int64_t n_vox, int32_t n_rot, const double* g, int64_t ld_g,
                   const int64_t* rotmat_inv, int64_t ld_rot, double scale, double* weight, void* workspace,
                   size_t workspace_bytes, void* stream);
JSCC_API int jscc_compton_project_f64(const float* records, const int32_t* row_id, int64_t n_ev, const float* coor,
                   int64_t n_vox, int32_t model, const void* eff, int32_t eff_dtype, int64_t ld_eff,
                   const double* img, double* f_out, void* stream);
JSCC_API int jscc_compton_backproject_f64(const float* records, const int32_t* row_id, int64_t n_ev,
                   const float* coor, int64_t n_vox, int32_t model, const void* eff, int32_t eff_dtype,
                   int64_t ld_eff, const double* g, double scale, double* weight, void* stream);
JSCC_API int jscc_rdp_prior_f64(const double* img, const int32_t* nbr, const float* weight, int64_t n_vox,
                   int32_t n_nbr, double gamma, double eps, double beta, double* value, double* grad,
                   int32_t accumulate, void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------ batched (multi-instance) SC path */

/*
 * BF16 GEMM on the tensor cores (tcgen05.mma, FP32 accumulation in tensor memory):
 *   out[m * ldo + n] = sum_{k < K} P[m * ldp + k] * R[n * ldr + k]     (m < M, n < nr <= 256)
 * P and R are BF16, both K-major (the K index contiguous); K, ldp and ldr multiples of 8;
 * P and R 16-byte aligned. k_splits > 1 splits K over CTAs (partials summed in a fixed order,
 * workspace jscc_bf16_gemm_workspace_bytes). For N instances sharing one SC matrix this is
 * the forward projection F = A_s X (P = subset rows of A, R = images) and the back projection
 * W = A_s^T Q (P = rows of a stored A^T restricted to the subset's bins, R = ratios): one pass
 * over A serves every instance (the per-instance passes of recon_osem_plane.py:28-30).
 */
JSCC_API size_t jscc_bf16_gemm_workspace_bytes(int64_t M, int32_t nr, int64_t K, int32_t k_splits);
JSCC_API int jscc_bf16_gemm_nt(const void* P, int64_t ldp, const void* R, int64_t ldr, int64_t M, int32_t nr,
                   int64_t K, int32_t k_splits, float* out, int64_t ldo, void* workspace,
                   size_t workspace_bytes, void* stream);

/*
 * Helpers of the batched OSEM step (instances n < n_inst, padded to np rows):
 *   jscc_batch_split:  xs[n][v] = bf16(x[n][v]), xs[np + n][v] = bf16(x[n][v] - xs[n][v])
 *                      (BF16 hi / lo pairs of FP32 images; rows n_inst..np-1 zero)
 *   jscc_batch_ratio:  f = F[b][n] + F[b][np + n] (clamped below at floor_v when use_floor);
 *                      q = y[n][b0 + b] / f; qs = hi / lo of q as above, [2 np x nb];
 *                      f_out[n][b] = f when non-NULL
 *   jscc_batch_weight: w_out[n][v] (+)= scale * (W[v][n] + W[v][np + n])
 */
JSCC_API int jscc_batch_split(const float* x, int64_t ldx, int32_t n_inst, int32_t np, int64_t V, void* xs,
                   int64_t ldxs, void* stream);
JSCC_API int jscc_batch_ratio(const float* F, int64_t ldf, const float* y, int64_t ldy, int64_t b0, int64_t nb,
                   int32_t n_inst, int32_t np, void* qs, int64_t ldqs, float* f_out, int64_t ldfo,
                   int32_t use_floor, float floor_v, void* stream);
JSCC_API int jscc_batch_weight(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np, float scale,
                   float* w_out, int64_t ldwo, int32_t accumulate, void* stream);

/*
 * Batched plain EM update (recon_osem_plane.py:54 per instance) from the back-projection GEMM:
 *   x[n][v] = x[n][v] * (W[v][n] + W[v][np + n]) / s_map[v]      (in place)
 * and, when xs is non-NULL, the updated images' BF16 hi / lo pairs as jscc_batch_split writes
 * them (rows n_inst..np-1 of xs are left as they are).
 */
JSCC_API int jscc_batch_em(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np, float* x,
                   int64_t ldx, const float* s_map, void* xs, int64_t ldxs, void* stream);

/*
 * Joint batched EM update (the joint loops' update per instance, recon_osem_plane.py:118 and
 * safe_em_update of recon_osem_plane_sparse.py:60-66):
 *   w = coef_a * (W[v][n] + W[v][np + n]) + coef_b * w_b[n][v]      (w_b may be NULL)
 *   JSCC_EM_PLAIN: x = x * w / s;  JSCC_EM_SAFE: nan/inf -> 0 in w and s, s > eps ? x max(w, 0) / s : 0
 * with s = s_map[n * lds + v] (lds = 0: one sensitivity for every instance), in place, and the
 * next hi / lo pair into xs when non-NULL.
 */
JSCC_API int jscc_batch_em_joint(const float* W, int64_t ldw, int64_t V, int32_t n_inst, int32_t np,
                   float coef_a, const float* w_b, int64_t ldwb, float coef_b, float* x, int64_t ldx,
                   const float* s_map, int64_t lds, int32_t mode, float eps, void* xs, int64_t ldxs,
                   void* stream);

/* Tensor-core GEMM waits that gave up since the last call (synchronous device read). */
JSCC_API int jscc_take_gemm_timeout_count(unsigned int* out);

/* ------------------------------------------------------------ MAP prior */

/*
 * Relative-difference prior (Nuyts et al. 2002) of img over a symmetric neighbour table,
 * value and gradient in one pass (the reference has no MAP path; this serves gradient-driven
 * reconstruction through the forward/adjoint projectors above):
 *   R(x) = 1/2 sum_j sum_{k in N(j)} w_jk (x_j - x_k)^2 / (x_j + x_k + gamma |x_j - x_k| + eps)
 * nbr / weight are neighbour-major [n_nbr, n_vox] (entry k * n_vox + j is the k-th neighbour
 * of voxel j, -1 = none); every edge must appear in both directions with the same weight.
 * value (may be NULL): *value += beta * R(x) (double, device memory; the caller zeroes it),
 * reduced in a fixed order (per-block sums in the workspace, then one block adds them in
 * order), so repeated calls give bit-identical values. The workspace (8-byte aligned, at least
 * jscc_rdp_prior_workspace_bytes(n_vox) bytes) is only needed when value is non-NULL.
 * grad  (may be NULL): grad[j] = (accumulate ? grad[j] : 0) + beta * dR/dx_j.
 * Out-of-range neighbour indices are skipped and counted (jscc_take_bad_index_count).
 */
JSCC_API size_t jscc_rdp_prior_workspace_bytes(int64_t n_vox);
JSCC_API int jscc_rdp_prior(const float* img, const int32_t* nbr, const float* weight, int64_t n_vox,
                   int32_t n_nbr, float gamma, float eps, float beta, double* value, float* grad,
                   int32_t accumulate, void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JSCC_GB300_H */
