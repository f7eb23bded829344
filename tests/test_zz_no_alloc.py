"""GPU test of jscc_sc_weight_noalloc, the SC weight entry point that allocates nothing.

It serves callers that cannot allocate device memory themselves (a host framework that
owns the GPU memory pool, an FFI caller without a device allocator, a loop that must not
pay cudaMalloc's synchronisation). Its scratch is a fixed 16 MiB array inside the
library. This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def _rot_args(rot, inv, n_rot):
    if rot is None:
        return None, None, 0
    return rot.data_ptr(), inv.data_ptr(), rot.stride(0)


def _call_with_workspace(lib, A, y, x, w, floor=None, rot=None, inv=None, n_rot=1):
    B, V = A.shape
    nbytes = lib.jscc_sc_weight_workspace_bytes(B, V, n_rot)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=A.device)
    rp, ip, ld_rot = _rot_args(rot, inv, n_rot)
    rc = lib.jscc_sc_weight(A.data_ptr(), 0 if A.dtype == torch.float32 else 1, A.stride(0), None, B, V,
                            y.data_ptr(), y.stride(0), n_rot, x.data_ptr(), rp, ip, ld_rot,
                            1 if floor is not None else 0, floor or 0.0, 1.0, w.data_ptr(), ws.data_ptr(),
                            nbytes, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.jscc_last_error()


def _call_noalloc(lib, A, y, x, w, floor=None, rot=None, inv=None, n_rot=1):
    B, V = A.shape
    rp, ip, ld_rot = _rot_args(rot, inv, n_rot)
    return lib.jscc_sc_weight_noalloc(A.data_ptr(), 0 if A.dtype == torch.float32 else 1, A.stride(0), None, B,
                                      V, y.data_ptr(), y.stride(0), n_rot, x.data_ptr(), rp, ip, ld_rot,
                                      1 if floor is not None else 0, floor or 0.0, 1.0, w.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)


def _problem(dev, B, V, seed, dtype=torch.float32):
    g = torch.Generator().manual_seed(seed)
    A = (torch.rand((B, V), generator=g) + 0.01).to(dtype).to(dev)
    y = (torch.rand((B, 1), generator=g) * 50).to(dev)
    x = (torch.rand((V, 1), generator=g) + 0.1).to(dev)
    return A, y, x


def test_noalloc_matches_workspace_entry_two_calls(cuda, lib):
    # two calls in a row with different sizes and dtypes: the shared scratch keeps the
    # first call's contents, which must not leak into the second call's result
    cases = [(_problem(cuda, 3000, 4800, 1), None), (_problem(cuda, 1024, 36000, 2, torch.bfloat16), 1e-12)]
    for (A, y, x), floor in cases:
        w_ref = torch.zeros((A.size(1), 1), device=cuda)
        _call_with_workspace(lib, A, y, x, w_ref, floor)
        w = torch.zeros_like(w_ref)
        assert _call_noalloc(lib, A, y, x, w, floor) == 0, lib.jscc_last_error()
        torch.cuda.synchronize()
        assert rel_l2(w.cpu(), w_ref.cpu()) < TOL_F32
    # the same problem twice more: identical results call after call
    A, y, x = cases[0][0]
    w1 = torch.zeros((A.size(1), 1), device=cuda)
    w2 = torch.zeros_like(w1)
    assert _call_noalloc(lib, A, y, x, w1) == 0
    assert _call_noalloc(lib, A, y, x, w2) == 0
    torch.cuda.synchronize()
    assert torch.equal(w1, w2)


def test_noalloc_rotation_blocks_after_direct_call(cuda, lib):
    """The rotated form (gather through rotmat, scatter back through rotmat_inv) with 8 and
    then 4 rotations per pass, straight after a one-rotation direct call: the scratch holds
    up to 8 rotated images and their partial sums, laid out differently for each rotation
    count, and what a larger call left behind must not leak into a smaller one."""
    from jscc_recon_spect_cylinder_gb300 import synthetic

    A1, y1, x1 = _problem(cuda, 2048, 4800, 3)
    w_ref = torch.zeros((4800, 1), device=cuda)
    _call_with_workspace(lib, A1, y1, x1, w_ref)
    w = torch.zeros_like(w_ref)
    assert _call_noalloc(lib, A1, y1, x1, w) == 0, lib.jscc_last_error()
    torch.cuda.synchronize()
    assert rel_l2(w.cpu(), w_ref.cpu()) < TOL_F32
    for views in (8, 4):
        prob = synthetic.sc_problem(n_r=40, n_theta=120, n_phi=1024, views=views, flat=False, total_counts=1e6)
        A = prob.sysmat.to(cuda)
        y = prob.proj.to(cuda).contiguous()          # [bins, views]: column r is view r
        rot, inv = prob.rotmat.to(cuda), prob.rotmat_inv.to(cuda)
        x = (torch.rand((A.size(1), 1), generator=torch.Generator().manual_seed(views)) + 0.1).to(cuda)
        assert lib.jscc_sc_weight_workspace_bytes(A.size(0), A.size(1), views) <= 16 * 1024 * 1024
        for floor in (None, 1e-12):
            w_ref = torch.zeros((A.size(1), 1), device=cuda)
            _call_with_workspace(lib, A, y, x, w_ref, floor, rot, inv, views)
            w1 = torch.zeros_like(w_ref)
            w2 = torch.zeros_like(w_ref)
            assert _call_noalloc(lib, A, y, x, w1, floor, rot, inv, views) == 0, lib.jscc_last_error()
            assert _call_noalloc(lib, A, y, x, w2, floor, rot, inv, views) == 0, lib.jscc_last_error()
            torch.cuda.synchronize()
            assert rel_l2(w1.cpu(), w_ref.cpu()) < TOL_F32
            assert torch.equal(w1, w2)


def test_noalloc_rejects_problems_beyond_scratch(cuda, lib):
    from jscc_recon_spect_cylinder_gb300 import _lib

    # 8 rotations over 400,000 voxels need far more than 16 MiB of scratch; the call is
    # rejected during argument checks, before any pointer is used or kernel launched
    B, V, R = 1000, 400000, 8
    assert lib.jscc_sc_weight_workspace_bytes(B, V, R) > 16 * 1024 * 1024
    dummy = torch.zeros(8, device=cuda)
    p = dummy.data_ptr()
    rc = lib.jscc_sc_weight_noalloc(p, 0, V, None, B, V, p, R, R, p, None, None, 0, 0, 0.0, 1.0, p,
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.JSCC_ERR_INVALID
    assert b"scratch" in lib.jscc_last_error()
