"""Multi-instance (batched) SC OSEM: N reconstructions that share one SC system matrix.

Each instance follows osem_bin_mode with one identity view (recon_osem_plane.py:45-61: per
subset, ``w = A_s^T (y_s / A_s x)``, ``x <- x * w / s_map``), but the N instances' projector
passes become two tensor-core GEMMs per subset (jscc_bf16_gemm_nt), so the matrix is streamed
from HBM once per pass for all instances:

    F  = A_s X          [bins_s x N]   (P = subset rows of A, R = images as BF16 hi / lo pairs)
    Q  = Y_s / F                        (jscc_batch_ratio, written as BF16 hi / lo pairs)
    W  = A_s^T Q        [V x N]        (P = the subset's columns of a stored A^T, R = Q)
    X <- X * W / s_map                  (jscc_batch_em, which also writes the next hi / lo pair)

Storage: A in BF16 with its rows permuted so that every subset is one contiguous block padded
to a multiple of 8 bins (zero rows), and the transpose of that matrix (both operands of both
GEMMs stay K-major): 2 x bins x V x 2 bytes. Instance vectors enter as hi / lo BF16 pairs
(~16 significant bits), so the error is that of the BF16 matrix, as in the single-instance
BF16 path. The K split of each GEMM shape is chosen by timing (``autotune``) and a whole
iteration over the subsets can be captured into a CUDA graph (``capture``).

BatchedJointOsem adds the Compton channel of the joint loops: each instance's own event list,
weighted through the fused cone kernels (all instances of a subset in one launch per direction,
jscc_compton_weight_batched with device segment tables), combined with the batched SC weights
in one safe EM update per subset; the whole iteration can be captured in one CUDA graph.
"""
from __future__ import annotations

import torch

from . import _lib, ops


def _pad8(n: int) -> int:
    return (n + 7) // 8 * 8


def subset_blocks(subsets):
    """Layout of the bin-permuted matrix: ``(blocks, perm)`` with one ``(row offset, bins,
    padded bins)`` block per subset (padded to a multiple of 8 rows, so every block and every
    column block of the transpose starts 16-byte aligned) and ``perm[row]`` = the reference's
    bin index held by that row (-1 on padding rows)."""
    blocks, off = [], 0
    for ids in subsets:
        nb = int(ids.numel())
        blocks.append((off, nb, _pad8(nb)))
        off += _pad8(nb)
    perm = torch.full((off,), -1, dtype=torch.int64)
    for (b0, nb, _), ids in zip(blocks, subsets):
        perm[b0:b0 + nb] = ids.to(torch.int64).cpu()
    return blocks, perm


class BatchedScOsem:
    """Batched plain SC OSEM over fixed subsets.

    sysmat:  [B, V] float32 / bfloat16 (any device; copied to ``device`` in BF16)
    subsets: list of 1-D bin-index tensors (the reference's split of a random permutation)
    s_map:   [V, 1] or [V] sensitivity shared by the instances
    n_inst:  number of instances (<= 128)
    """

    F_SPLITS = (1, 2, 3, 4, 6, 8)
    B_SPLITS = (1, 2, 4)

    def __init__(self, sysmat, subsets, s_map, n_inst, device="cuda"):
        dev = torch.device(device)
        if dev.type != "cuda":
            raise RuntimeError("BatchedScOsem runs on CUDA only (there is no CPU fallback)")
        if not 1 <= n_inst <= 128:
            raise ValueError(f"n_inst = {n_inst} outside [1, 128]")
        B, V = sysmat.shape
        if V % 8:
            raise ValueError(f"the voxel count ({V}) must be a multiple of 8")
        self.dev, self.V, self.B, self.n = dev, V, B, n_inst
        self.np = _pad8(n_inst)
        self.nr = 2 * self.np
        self.blocks, perm = subset_blocks(subsets)  # (row offset, real bins, padded bins) per subset
        self.B_pad = perm.numel()
        A = torch.zeros((self.B_pad, V), dtype=torch.bfloat16, device=dev)
        for (b0, nb, _), ids in zip(self.blocks, subsets):
            ids = ids.to(torch.int64).cpu()
            A[b0:b0 + nb] = sysmat[ids.to(sysmat.device)].to(dev, torch.bfloat16)
        self.perm = perm.to(dev)
        self.A = A
        self.AT = A.t().contiguous()
        self.s_map = s_map.reshape(-1).to(dev, torch.float32).contiguous()
        if self.s_map.numel() != V:
            raise ValueError("s_map must have one entry per voxel")
        # working buffers (fixed addresses: a captured graph reads and writes them)
        self.X = torch.zeros((n_inst, V), dtype=torch.float32, device=dev)
        self.Y = torch.zeros((n_inst, self.B_pad), dtype=torch.float32, device=dev)
        self.Xs = torch.zeros((self.nr, V), dtype=torch.bfloat16, device=dev)
        nb_max = max(b[2] for b in self.blocks)
        self.F = torch.empty((nb_max, self.nr), dtype=torch.float32, device=dev)
        self.Qs = [torch.zeros((self.nr, nbp), dtype=torch.bfloat16, device=dev) for _, _, nbp in self.blocks]
        self.W = torch.empty((V, self.nr), dtype=torch.float32, device=dev)
        self.splits = {}
        self.graph = None
        self.graph_launches = 0
        self.floor = None  # clamp_min of the forward projection (joint local loops: 1e-12)

    # ------------------------------------------------------------------ data
    def set_projections(self, proj):
        """proj [n_inst, B] (the reference's bin order) -> the permuted, padded copy."""
        p = proj.to(self.dev, torch.float32)
        if p.shape != (self.n, self.B):
            raise ValueError(f"projections must be [{self.n}, {self.B}]")
        self.Y.zero_()
        real = self.perm >= 0
        self.Y[:, real] = p[:, self.perm[real]]

    def set_images(self, img):
        """img [n_inst, V] float32 (copied into the batch)."""
        self.X.copy_(img.to(self.dev, torch.float32).reshape(self.n, self.V))

    # ------------------------------------------------------------------ kernels
    def _gemm(self, P, R, out, key):
        return ops.bf16_gemm_nt(P, R, out=out, k_splits=self.splits.get(key, 1))

    def _subset(self, k):
        b0, nb, nbp = self.blocks[k]
        lib = _lib.load()
        st = _lib.stream_handle(self.dev)
        F = self.F[:nbp]
        self._gemm(self.A[b0:b0 + nbp], self.Xs, F, ("f", nbp))
        _lib.check(lib.jscc_batch_ratio(F.data_ptr(), F.stride(0), self.Y.data_ptr(), self.Y.stride(0), b0, nb, self.n,
                                        self.np, self.Qs[k].data_ptr(), self.Qs[k].stride(0), None, 0,
                                        1 if self.floor is not None else 0,
                                        float(self.floor) if self.floor is not None else 0.0, st),
                   "jscc_batch_ratio")
        self._gemm(self.AT[:, b0:b0 + nbp], self.Qs[k], self.W, ("b", nbp))
        _lib.check(lib.jscc_batch_em(self.W.data_ptr(), self.W.stride(0), self.V, self.n, self.np, self.X.data_ptr(),
                                     self.X.stride(0), self.s_map.data_ptr(), self.Xs.data_ptr(), self.Xs.stride(0),
                                     st), "jscc_batch_em")

    def _iteration(self):
        lib = _lib.load()
        _lib.check(lib.jscc_batch_split(self.X.data_ptr(), self.X.stride(0), self.n, self.np, self.V,
                                        self.Xs.data_ptr(), self.Xs.stride(0), _lib.stream_handle(self.dev)),
                   "jscc_batch_split")
        for k in range(len(self.blocks)):
            self._subset(k)

    def iterate(self, n_iter=1):
        """n_iter OSEM iterations (every subset once each) of all instances, in place."""
        for _ in range(n_iter):
            if self.graph is not None:
                self.graph.replay()
                _lib.load().jscc_count_graph_launches(self.graph_launches)
            else:
                self._iteration()
        return self.X

    # ------------------------------------------------------------------ tuning and capture
    def autotune(self, reps=3):
        """Choose the K split of each GEMM shape by timing the candidates on the current
        images and projections (results are recomputed afterwards, state is unchanged)."""
        saved = self.X.clone()
        lib = _lib.load()
        _lib.check(lib.jscc_batch_split(self.X.data_ptr(), self.X.stride(0), self.n, self.np, self.V,
                                        self.Xs.data_ptr(), self.Xs.stride(0), _lib.stream_handle(self.dev)),
                   "jscc_batch_split")
        firsts = {}
        for k, (_, _, nbp) in enumerate(self.blocks):
            firsts.setdefault(nbp, k)
        for kind, cands in (("f", self.F_SPLITS), ("b", self.B_SPLITS)):
            for nbp, k in firsts.items():
                b0 = self.blocks[k][0]
                key = (kind, nbp)
                best = None
                for s in cands:
                    self.splits[key] = s
                    P, R, out = ((self.A[b0:b0 + nbp], self.Xs, self.F[:nbp]) if kind == "f"
                                 else (self.AT[:, b0:b0 + nbp], self.Qs[k], self.W))
                    self._gemm(P, R, out, key)  # warm-up (workspace, attributes)
                    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    t0.record()
                    for _ in range(reps):
                        self._gemm(P, R, out, key)
                    t1.record()
                    torch.cuda.synchronize(self.dev)
                    ms = t0.elapsed_time(t1) / reps
                    if best is None or ms < best[0]:
                        best = (ms, s)
                self.splits[key] = best[1]
        self.X.copy_(saved)
        return dict(self.splits)

    def capture(self):
        """Capture one iteration (split + every subset) into a CUDA graph; ``iterate`` then
        replays it. Call after ``autotune`` (or one eager iteration) so that workspaces and
        kernel attributes exist before capture."""
        saved = self.X.clone()
        self._iteration()  # warm-up outside the capture
        torch.cuda.synchronize(self.dev)
        self.X.copy_(saved)
        g = torch.cuda.CUDAGraph()
        n0 = _lib.launch_count()
        with torch.cuda.graph(g):
            self._iteration()
        self.graph_launches = _lib.launch_count() - n0  # kernels one replay launches
        self.graph = g
        return g


def osem_bin_mode_batched(sysmat, proj, img, s_map, subsets, iterations, graph=True, tune=True):
    """Batched form of osem_bin_mode for N instances with one identity view:
    ``proj`` [N, B], ``img`` [N, V] (initial images), ``subsets`` the bin-index split.
    Returns the images after ``iterations`` OSEM iterations, [N, V] float32."""
    b = BatchedScOsem(sysmat, subsets, s_map, proj.size(0), device=img.device if img.is_cuda else "cuda")
    b.set_projections(proj)
    b.set_images(img)
    if tune:
        b.autotune()
    if graph:
        b.capture()
    return b.iterate(iterations).clone()


class BatchedJointOsem(BatchedScOsem):
    """Batched joint JSCCSD OSEM: per instance, every subset update is
    ``w = alpha w_SC + (2 - alpha) w_C`` and ``x <- safe_em_update(x, w, s_joint)`` with the SC
    forward projection floored at 1e-12 (osem_joint_mode_local_sparse,
    recon_osem_local_sparse_jsccsd_only.py:58-100). The SC weights of all instances come from
    the tensor-core GEMMs; each instance's Compton weight ``T^T (1 / T x)`` over its own events
    of the subset comes from the fused cone kernels (T recomputed, nothing stored per event but
    its 64-byte record), with the batch's BF16 matrix as the efficiency rows. With the strict
    model, every subset's events of all instances form one ops.ComptonBatch (one forward and
    one back launch for the whole batch, partial images summed per instance in a fixed order);
    other models go instance by instance through ops.compton_weight.

    events:  per instance, per subset, a ComptonEvents block (row ids in the reference's bin order)
    coor:    [V, 3] voxel centres on the device
    s_joint: [n_inst, V] per-instance joint sensitivities
    """

    def __init__(self, sysmat, subsets, s_joint, events, coor, alpha=0.5, device="cuda"):
        n_inst = len(events)
        s_joint = s_joint.reshape(n_inst, -1)
        super().__init__(sysmat, subsets, s_joint[0], n_inst, device=device)
        if any(len(ev_n) != len(self.blocks) for ev_n in events):
            raise ValueError("events must hold one block per subset for every instance")
        self.floor = 1e-12
        self.alpha = float(alpha)
        self.S = s_joint.to(self.dev, torch.float32).contiguous()
        self.coor = coor.to(self.dev, torch.float32).contiguous()
        inv = torch.full((self.B,), -1, dtype=torch.int64, device=self.dev)
        real = self.perm >= 0
        inv[self.perm[real]] = torch.arange(self.B_pad, device=self.dev)[real]
        self.events = []  # (records, row ids into the permuted matrix, model) per instance and subset
        for ev_n in events:
            per = []
            for ev in ev_n:
                rid = inv[ev.row_id.to(self.dev, torch.int64)].to(torch.int32).contiguous() if len(ev) else ev.row_id
                per.append((ev.records, rid, ev.model))
            self.events.append(per)
        self.WC = torch.zeros((n_inst, self.V), dtype=torch.float32, device=self.dev)
        self.cbatch = None
        if all(m == _lib.CONE_STRICT for per in self.events for _, _, m in per):
            self.cbatch = [ops.ComptonBatch([(per[k][0], per[k][1]) for per in self.events], self.V, self.dev)
                           for k in range(len(self.blocks))]
            self.events = None  # the batches hold their own (sorted, padded) copies

    def _subset(self, k):
        b0, nb, nbp = self.blocks[k]
        lib = _lib.load()
        st = _lib.stream_handle(self.dev)
        F = self.F[:nbp]
        self._gemm(self.A[b0:b0 + nbp], self.Xs, F, ("f", nbp))
        _lib.check(lib.jscc_batch_ratio(F.data_ptr(), F.stride(0), self.Y.data_ptr(), self.Y.stride(0), b0, nb, self.n,
                                        self.np, self.Qs[k].data_ptr(), self.Qs[k].stride(0), None, 0, 1, self.floor,
                                        st), "jscc_batch_ratio")
        self._gemm(self.AT[:, b0:b0 + nbp], self.Qs[k], self.W, ("b", nbp))
        self.WC.zero_()
        if self.cbatch is not None:
            self.cbatch[k].weight(self.X, self.A, self.coor, out=self.WC)
        else:
            for n in range(self.n):
                rec, rid, model = self.events[n][k]
                if rec.size(0):
                    ops.compton_weight(rec, rid, self.coor, self.X[n], model=model, eff=self.A, out=self.WC[n])
        _lib.check(lib.jscc_batch_em_joint(self.W.data_ptr(), self.W.stride(0), self.V, self.n, self.np, self.alpha,
                                           self.WC.data_ptr(), self.WC.stride(0), 2.0 - self.alpha, self.X.data_ptr(),
                                           self.X.stride(0), self.S.data_ptr(), self.S.stride(0), _lib.EM_SAFE, 1e-12,
                                           self.Xs.data_ptr(), self.Xs.stride(0), st), "jscc_batch_em_joint")
