"""GPU parity of the Compton cone kernel (a) and the sparse coarse<->fine kernels (c)
against the reference's golden outputs and the oracle.

Tolerances: cone rows are compared per row relative to the row maximum (float32 acos /
exp / sqrt in a different operation order than torch: <= 2e-5 strict, <= 1e-4 legacy);
weights and images by relative L2 <= 1e-5 (FP32 path)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import compton as oc
from oracle import sparse as osp

pytestmark = pytest.mark.gpu

TOL_ROW = 2e-5
TOL_ROW_LEGACY = 1e-4
TOL_W = 1e-5


def _rows_close(a, b, rtol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-30)
    err = np.abs(a - b) / scale
    assert err.max() < rtol, err.max()


def _args(g, tag):
    return [float(v) for v in g[f"{tag}_args"]]


@pytest.mark.parametrize("tag", ["planar", "cyl"])
def test_strict_builder_golden(cuda, golden, tag):
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls

    g = golden("compton_builders")
    dr1, dr2, e0, res, tmax, tmin, tsum = _args(g, tag)
    L = torch.from_numpy(g[f"{tag}_smeared"]).to(cuda)
    t, tc, ts, _ = pls.build_rows_from_smeared(torch.from_numpy(g[f"{tag}_sysmat"]).to(cuda),
                                               torch.from_numpy(g[f"{tag}_det"]).to(cuda),
                                               torch.from_numpy(g["coor"]).to(cuda), L, dr1, dr2, e0, res, tmax,
                                               tmin, tsum)
    _rows_close(t.cpu(), g[f"{tag}_t"], TOL_ROW)
    _rows_close(tc.cpu(), g[f"{tag}_tc"], TOL_ROW)
    _rows_close(ts.cpu(), g[f"{tag}_ts"], 1e-6)


@pytest.mark.parametrize("tag", ["planar", "cyl"])
def test_strict_builder_wrapper_smears_in_place(cuda, golden, tag):
    """The reference's contract: the caller's list is smeared in place with CPU torch.randn
    draws; outputs are CPU tensors. GPU float32 arithmetic can round the smeared energies
    differently from the CPU by 1 ulp, so values are compared with a tolerance."""
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls

    g = golden("compton_builders")
    a = _args(g, tag)
    L = torch.from_numpy(g[f"{tag}_list"].copy()).to(cuda)
    torch.manual_seed(77)
    t, tc, ts = pls.get_compton_backproj_list_single(torch.from_numpy(g[f"{tag}_sysmat"]).to(cuda),
                                                     torch.from_numpy(g[f"{tag}_det"]).to(cuda),
                                                     torch.from_numpy(g["coor"]).to(cuda), L, *a, cuda)
    assert t.device.type == "cpu"
    np.testing.assert_allclose(L.cpu().numpy(), g[f"{tag}_smeared"], rtol=3e-7, atol=0)
    assert t.shape == g[f"{tag}_t"].shape
    _rows_close(t, g[f"{tag}_t"], 1e-4)


@pytest.mark.parametrize("tag", ["planar", "cyl"])
def test_legacy_builder_golden(cuda, golden, tag):
    from jscc_recon_spect_cylinder_gb300 import _lib
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls

    g = golden("compton_builders")
    dr, e0, res, tmax, tmin, tsum = 1.0 + _args(g, tag)[0], *_args(g, tag)[2:]
    L = torch.from_numpy(g[f"{tag}_legacy_smeared"]).to(cuda)
    t, tc, ts, _ = pls.build_rows_from_smeared(torch.from_numpy(g[f"{tag}_sysmat"]).to(cuda),
                                               torch.from_numpy(g[f"{tag}_det"]).to(cuda),
                                               torch.from_numpy(g["coor"]).to(cuda), L, dr, dr, e0, res, tmax, tmin,
                                               tsum, model=_lib.CONE_LEGACY, stability=False)
    _rows_close(t.cpu(), g[f"{tag}_legacy_t"], TOL_ROW_LEGACY)
    _rows_close(tc.cpu(), g[f"{tag}_legacy_tc"], TOL_ROW_LEGACY)


def _cone_problem(cuda, n_events=3000, n_r=20, n_theta=72, seed=4):
    """Cylinder detector (isotropic sigma_pos with delta_r = 0.8 mm), 511 keV events."""
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(n_r, n_theta, 40.0)
    scat = synthetic.cylinder_pixels(120.0, 32, 4, 3.0)
    absb = synthetic.cylinder_pixels(150.0, 32, 4, 3.0)
    det = torch.cat((scat, absb)).float()
    g = torch.Generator().manual_seed(seed)
    sysmat = torch.rand((det.size(0), grid.n_vox), generator=g) * 1e-3 + 1e-5
    rng = np.random.default_rng(seed)
    e0 = 0.511
    cp1 = rng.integers(1, scat.size(0) + 1, n_events)
    cp2 = rng.integers(scat.size(0) + 1, det.size(0) + 1, n_events)
    e1 = rng.uniform(0.08, 0.3, n_events)
    L = np.stack((cp1, e1, cp2, e0 - e1), axis=1).astype(np.float32)
    res = 0.1 * (0.662 / e0) ** 0.5
    args = (0.8, 0.8, e0, res, 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001, 0.05, e0 - 0.06)
    return grid, det, sysmat, L, args


def test_fused_cone_weight_matches_stored_t(cuda):
    """The fused on-the-fly weight equals T^T(1/(Tx)) over the builder's stored rows
    (row normalisation does not change the list-mode weight), with every pair evaluated
    (the default) and with the 9-sigma window, which changes it by far less than float32
    rounding."""
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    grid, det, sysmat, L, args = _cone_problem(cuda)
    Ld = torch.from_numpy(L).to(cuda)
    A = sysmat.to(cuda)
    coor = grid.coor.to(cuda)
    t, _, _, kept = pls.build_rows_from_smeared(A, det.to(cuda), coor, Ld, *args)
    ev = pls.get_compton_event_params(A, det.to(cuda), coor, Ld, *args, theta_fp64=False, window_sigmas=9.0)
    assert torch.equal(ev.list_index, kept)  # identical event selection incl. row filters
    x = torch.rand((grid.n_vox, 1), generator=torch.Generator().manual_seed(1)).to(cuda) + 0.5
    w_stored = rop.get_weight_compton(t, x)
    w_fused = rop.get_weight_compton_fused(ev, coor, A, x, use_window=True)
    w_exact = rop.get_weight_compton_fused(ev, coor, A, x)  # every pair (the default)
    assert rel_l2(w_exact.cpu(), w_stored.cpu()) < TOL_W
    assert rel_l2(w_fused.cpu(), w_stored.cpu()) < TOL_W
    assert rel_l2(w_fused.cpu(), w_exact.cpu()) < 1e-6
    # against the float32 oracle (the reference's arithmetic, pinned by the golden tests)
    # on the same events. Float32 and float64 evaluations of the reference's formula differ
    # by ~2e-3 here: where the voxel, the first and the second hit are nearly collinear
    # (beta ~ 180 deg) 1 - cos^2(beta) cancels to its 1e-12 clamp in float32 and sigma_pos
    # explodes (process_list_plane_strict.py:113-114); the kernel reproduces the reference.
    from oracle import osem_sc

    ids = ev.list_index.cpu().numpy()
    cp1, cp2 = L[ids, 0].astype(np.int64), L[ids, 2].astype(np.int64)
    d = det.numpy()
    tc32 = oc.cone_rows_strict(d[cp1 - 1], d[cp2 - 1], L[ids, 1], oc.pos_sigma_sq(d, args[0])[cp1 - 1],
                               oc.pos_sigma_sq(d, args[1])[cp2 - 1], grid.coor.numpy(), args[2], args[3],
                               dtype=np.float32)
    w32 = osem_sc.get_weight_compton(tc32 * sysmat.numpy()[cp1 - 1], x.cpu().numpy(), dtype=np.float32)
    assert rel_l2(w_fused.cpu(), w32) < TOL_W
    assert rel_l2(w_exact.cpu(), w32) < TOL_W


def test_fused_list_mode_osem_with_rotations(cuda):
    """osem_list_mode over stored T and osem_list_mode_fused over event records agree
    (rotated views, 2 subsets x 2 divides)."""
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid, det, sysmat, L, args = _cone_problem(cuda, n_events=2400)
    R, S, D = 4, 2, 2
    rot, inv = synthetic.cyclic_rotation_tables(grid.n_r, grid.n_theta, R)
    rot, inv = rot.to(cuda), inv.to(cuda)
    A, coor, detc = sysmat.to(cuda), grid.coor.to(cuda), det.to(cuda)
    chunks = torch.chunk(torch.from_numpy(L).to(cuda), R)
    t_list = [[[[None] for _ in range(D)] for _ in range(R)] for _ in range(S)]
    e_list = [[[[None] for _ in range(D)] for _ in range(R)] for _ in range(S)]
    for r in range(R):
        t, _, _, _ = pls.build_rows_from_smeared(A, detc, coor, chunks[r].contiguous(), *args)
        ev = pls.get_compton_event_params(A, detc, coor, chunks[r].contiguous(), *args, theta_fp64=False)
        assert len(ev) == t.size(0)
        for j, (ts, es) in enumerate(zip(rop.split_tensor_even(t, S), ev.split(S))):
            for k, (tk, ek) in enumerate(zip(rop.split_tensor_even(ts, D), es.split(D))):
                t_list[j][r][k][0] = tk
                e_list[j][r][k][0] = ek
    s_d = torch.rand((grid.n_vox, 1), generator=torch.Generator().manual_seed(2)).to(cuda) + 0.5
    x0 = torch.ones((grid.n_vox, 1), device=cuda)
    img_t = rop.osem_list_mode(t_list, [rot], [inv], x0, s_d, R)
    img_f = rop.osem_list_mode_fused(e_list, [coor], [A], [rot], [inv], x0, s_d, R)
    assert rel_l2(img_f.cpu(), img_t.cpu()) < TOL_W


def test_row_stats_match_oracle(cuda):
    from jscc_recon_spect_cylinder_gb300 import _compton, _lib, ops

    grid, det, sysmat, L, args = _cone_problem(cuda, n_events=500)
    Ld = torch.from_numpy(L).to(cuda)
    idx, rec, rid = _compton.select_events(Ld, det.to(cuda), args[0], args[1], *args[2:], theta_fp64=False)
    ref_idx = oc.event_filter(L, det.numpy(), args[2], args[4], args[5], args[6])
    np.testing.assert_array_equal(idx.cpu().numpy(), ref_idx)
    s1, s2, nan = ops.compton_row_stats(rec, rid, grid.coor.to(cuda), model=_lib.CONE_STRICT, eff=sysmat.to(cuda))
    cp1 = L[ref_idx, 0].astype(np.int64)
    cp2 = L[ref_idx, 2].astype(np.int64)
    d = det.numpy()
    tc = oc.cone_rows_strict(d[cp1 - 1], d[cp2 - 1], L[ref_idx, 1], oc.pos_sigma_sq(d, args[0])[cp1 - 1],
                             oc.pos_sigma_sq(d, args[1])[cp2 - 1], grid.coor.numpy(), args[2], args[3],
                             dtype=np.float32)
    t = tc * sysmat.numpy()[cp1 - 1]
    assert rel_l2(s1.cpu(), t.sum(1)) < 1e-5
    assert rel_l2(s2.cpu(), (t.astype(np.float64) ** 2).sum(1)) < 1e-5
    assert not nan.any()


def test_bad_detector_ids_are_dropped_and_counted(cuda):
    from jscc_recon_spect_cylinder_gb300 import _compton, _lib

    grid, det, sysmat, L, args = _cone_problem(cuda, n_events=64)
    L = L.copy()
    L[3, 0] = det.size(0) + 5
    L[7, 2] = 0
    _lib.take_bad_detector_count()
    idx, _, _ = _compton.select_events(torch.from_numpy(L).to(cuda), det.to(cuda), args[0], args[1], *args[2:])
    torch.cuda.synchronize()
    assert 3 not in idx.tolist() and 7 not in idx.tolist()
    assert _lib.take_bad_detector_count() >= 1  # counted when the event passed the energy tests


def test_empty_and_fully_filtered_lists(cuda):
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_sparse as psp
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    grid, det, sysmat, L, args = _cone_problem(cuda, n_events=10)
    A, detc, coor = sysmat.to(cuda), det.to(cuda), grid.coor.to(cuda)
    empty = torch.zeros((0, 4), device=cuda)
    t, tc, ts, idx = pls.build_rows_from_smeared(A, detc, coor, empty, *args)
    assert t.shape == (0, grid.n_vox)
    L2 = torch.from_numpy(L).to(cuda)
    L2[:, 1] = 5.0  # above every threshold: nothing survives
    t, _, _, _ = pls.build_rows_from_smeared(A, detc, coor, L2, *args)
    assert t.shape == (0, grid.n_vox)
    p = cso.build_compton_sparse_projector(grid.coor, 2, 1)
    rows = psp.build_sparse_rows_from_smeared(A, detc, p, L2, *args)
    assert rows.shape == (0, p.coarse_pixel_num + 1)


# ----------------------------------------------------------------------------- sparse kernels
def _r10(cuda, g):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    return cso.build_compton_sparse_projector(torch.from_numpy(g["r10_coor_full"]), 2, 2, 10)


def test_sparse_operators_golden_r10(cuda, golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    g = golden("sparse_ops")
    p = _r10(cuda, g).to(cuda)
    rc = torch.from_numpy(g["r10_rows_c"]).to(cuda)
    rf = torch.from_numpy(g["r10_rows_f"]).to(cuda)
    np.testing.assert_allclose(cso.upsample_coarse_rows_to_fine(rc, p).cpu(), g["r10_up"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(cso.project_fine_rows_to_coarse_adjoint(rf, p).cpu(), g["r10_adj"], rtol=1e-5,
                               atol=1e-6)
    np.testing.assert_allclose(cso.reduce_fine_rows_to_coarse(rf, p).cpu(), g["r10_red"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(cso.reduce_fine_image_to_coarse(torch.from_numpy(g["r10_img_f"]).to(cuda), p).cpu(),
                               g["r10_img_red"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(
        cso.upsample_coarse_weight_to_fine(torch.from_numpy(g["r10_img_c"]).to(cuda), p).cpu(), g["r10_img_up"],
        rtol=1e-6, atol=1e-7)


def test_upsample_adjoint_identity_full_size(cuda):
    """<U c, f> = <c, U^T f> on a config-3-size grid (100 x 360, theta stride 4): a
    size-independent property of the pair (float32 accumulation, float64 dot products)."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(100, 360, 100.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1).to(cuda)
    assert p.coarse_pixel_num == 9000
    g = torch.Generator(device=cuda).manual_seed(7)
    c = torch.rand((64, p.coarse_pixel_num), device=cuda, generator=g)
    f = torch.rand((64, p.fine_pixel_num), device=cuda, generator=g)
    lhs = (cso.upsample_coarse_rows_to_fine(c, p).double() * f.double()).sum()
    rhs = (c.double() * cso.project_fine_rows_to_coarse_adjoint(f, p).double()).sum()
    assert abs((lhs - rhs) / lhs).item() < 1e-6


def test_pack_unpack_golden(cuda, golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    g = golden("sparse_ops")
    rows = torch.from_numpy(g["s_event_rows"]).to(cuda)
    cp1, tc = cso.unpack_sparse_event_rows(rows)
    np.testing.assert_array_equal(cp1.cpu().numpy(), np.round(g["s_event_rows"][:, 0]).astype(np.int64))
    packed = cso.pack_sparse_event_rows(cp1, tc.contiguous())
    assert torch.equal(packed, rows)


def test_sparse_builder_and_weights_golden(cuda, golden):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_sparse as psp
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_sparse_jsccsd_only as loc
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane_sparse as rsp

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), 4, 2, 4).to(cuda)
    A = torch.from_numpy(g["s_sysmat"]).to(cuda)
    a = [float(v) for v in g["s_args"]]
    rows = psp.build_sparse_rows_from_smeared(A, torch.from_numpy(g["s_det"]).to(cuda), p,
                                              torch.from_numpy(g["s_smeared"]).to(cuda), *a)
    ref = g["s_event_rows"]
    np.testing.assert_array_equal(rows[:, 0].cpu().numpy(), ref[:, 0])
    _rows_close(rows[:, 1:].cpu(), ref[:, 1:], TOL_ROW)
    R = torch.from_numpy(ref).to(cuda)
    t_fine, valid = cso.materialize_sparse_event_rows_to_fine(R, A, p)
    np.testing.assert_array_equal(valid.cpu().numpy(), g["s_valid"])
    _rows_close(t_fine.cpu(), g["s_t_fine"], 1e-5)
    x = torch.from_numpy(g["s_x"]).to(cuda)
    assert rel_l2(rsp.get_weight_compton_sparse(R, A, x, p).cpu(), g["s_w_grouped"]) < TOL_W
    assert rel_l2(loc.get_weight_compton_sparse(R, A, x, p).cpu(), g["s_w_mat"]) < TOL_W
    # host-resident block (the reference's pinned spill) is copied first
    assert rel_l2(rsp.get_weight_compton_sparse(R.cpu(), A, x, p).cpu(), g["s_w_grouped"]) < TOL_W


def test_sparse_osem_loops_vs_oracle(cuda, golden):
    """osem_list_mode_sparse / osem_joint_mode_sparse / osem_joint_mode_local_sparse against
    the FP64 oracle on the golden sparse problem (2 subsets, 1 rotation)."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_sparse_jsccsd_only as loc
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane_sparse as rsp
    from oracle import osem_sc

    g = golden("sparse_ops")
    pn = osp.build_projector(g["s_coor"], 4, 2, 4)
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), 4, 2, 4).to(cuda)
    A = torch.from_numpy(g["s_sysmat"]).to(cuda)
    rows = g["s_event_rows"]
    V = A.size(1)
    halves = [rows[: rows.shape[0] // 2], rows[rows.shape[0] // 2:]]
    t_list = [[[[torch.from_numpy(h).to(cuda)]]] for h in halves]
    ident = torch.arange(1, V + 1, device=cuda).unsqueeze(1)
    s = torch.from_numpy(g["s_x"]).to(cuda) + 1.0
    x0 = torch.ones((V, 1), device=cuda)
    img = rsp.osem_list_mode_sparse(t_list, [A], [p], [ident], [ident], x0, s, 1)
    ref = np.ones((V, 1))
    for h in halves:
        ref = osem_sc.safe_em_update(ref, osp.weight_grouped(h, g["s_sysmat"], ref, pn), s.cpu().numpy())
    assert rel_l2(img.cpu(), ref) < TOL_W
    # joint local form: alpha * w_s + (2 - alpha) * w_c, materialise semantics
    B = A.size(0)
    y = torch.poisson(A @ torch.ones((V, 1), device=cuda) * 50)
    sub = [torch.arange(0, B // 2, device=cuda), torch.arange(B // 2, B, device=cuda)]
    img = loc.osem_joint_mode_local_sparse([[A[i]] for i in sub], [[y[i]] for i in sub], t_list, [A], [p], [ident],
                                           [ident], x0, s, 0.5, 1, cuda)
    ref = np.ones((V, 1))
    An, yn = g["s_sysmat"], y.cpu().numpy()
    for i, h in zip(sub, halves):
        ic = i.cpu().numpy()
        w = 0.5 * osem_sc.get_weight_single(An[ic], yn[ic], ref, floor=1e-12) + \
            1.5 * osp.weight_materialize(h, An, ref, pn)
        ref = osem_sc.safe_em_update(ref, w, s.cpu().numpy())
    assert rel_l2(img.cpu(), ref) < TOL_W


@pytest.mark.parametrize("grouped", [False, True])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_grouped_kernel_matches_event_kernel(cuda, golden, grouped, dtype):
    """The grouped coarse-space kernel and the per-event fine-space kernel compute the same
    weight (packed and split storage, both semantics, rotated view, FP32 and BF16 rows)."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops, synthetic

    g = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(g["s_coor"]), 4, 2, 4)
    tb = cso.tables(p, cuda)
    A = torch.from_numpy(g["s_sysmat"]).to(cuda)
    rows = torch.from_numpy(g["s_event_rows"]).to(cuda)
    rows = torch.cat([rows] * 7)  # repeated first-hit rows -> real groups
    V = A.size(1)
    x = torch.from_numpy(g["s_x"]).to(cuda)
    w_ev = ops.sparse_weight(rows, A, tb, x, grouped=grouped, method="event")
    w_gr = ops.sparse_weight(rows, A, tb, x, grouped=grouped)
    assert rel_l2(w_gr.cpu(), w_ev.cpu()) < TOL_W
    ids, tc = ops.split_sparse_rows(rows, dtype)
    w_sp_ev = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped, method="event")
    w_sp_gr = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped)
    assert rel_l2(w_sp_gr.cpu(), w_sp_ev.cpu()) < TOL_W
    # rotated view: 24 theta per ring, 4 views of 6 steps
    rot, inv = synthetic.cyclic_rotation_tables(6 * 4, 24, 4)
    rot, inv = rot.to(cuda), inv.to(cuda)
    a = ops.sparse_weight(rows, A, tb, x, grouped=grouped, rotmat=rot, rotmat_inv=inv, rot_col=2, method="event")
    b = ops.sparse_weight(rows, A, tb, x, grouped=grouped, rotmat=rot, rotmat_inv=inv, rot_col=2)
    assert rel_l2(b.cpu(), a.cpu()) < TOL_W
    # deterministic
    assert torch.equal(ops.sparse_weight(rows, A, tb, x, grouped=grouped), w_gr)


@pytest.mark.parametrize("theta_stride", [2, 4, 8])
def test_grouped_kernel_tap_widths(cuda, theta_stride):
    """One-plane grids whose adjoint tap width K = 2 * stride - 1 (3, 7, 15) takes each of
    the kernel's compile-time widths (4, 8) and the runtime-width path."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops, synthetic

    grid = synthetic.polar_grid(12, 72, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, theta_stride, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    assert tb.adj_width == 2 * theta_stride - 1
    g = torch.Generator().manual_seed(theta_stride)
    n_det = 50
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(cuda)
    n = 4000
    tc = torch.rand((n, p.coarse_pixel_num), generator=g) ** 3
    cp1 = torch.randint(1, n_det + 1, (n,), generator=g)
    rows = torch.cat((cp1.float().unsqueeze(1), tc), dim=1).to(cuda)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    for grouped in (False, True):
        w_ev = ops.sparse_weight(rows, A, tb, x, grouped=grouped, method="event")
        w_gr = ops.sparse_weight(rows, A, tb, x, grouped=grouped)
        assert rel_l2(w_gr.cpu(), w_ev.cpu()) < TOL_W
        ids, tcb = ops.split_sparse_rows(rows, torch.bfloat16)
        a = ops.sparse_weight_split(ids, tcb, A.to(torch.bfloat16), tb, x, grouped=grouped, method="event")
        b = ops.sparse_weight_split(ids, tcb, A.to(torch.bfloat16), tb, x, grouped=grouped)
        assert rel_l2(b.cpu(), a.cpu()) < TOL_W


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("n_det,n_events", [(400, 3000), (30, 2000), (700, 700)])
def test_grouped_bulk_pipeline(cuda, dtype, n_det, n_events):
    """Split rows with 16-byte aligned starts and lengths take the bulk-copy pipeline: groups
    larger than a batch (several batches per group), more groups than CTAs (batches
    prefetched across group boundaries) and one-event groups all match the per-event
    kernel, both semantics, and no device wait gives up."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, synthetic
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    grid = synthetic.polar_grid(16, 96, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    vc = p.coarse_pixel_num
    assert (vc * 2) % 16 == 0 and (grid.n_vox * 2) % 16 == 0
    g = torch.Generator().manual_seed(n_det + n_events)
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(cuda).to(dtype)
    tc = (torch.rand((n_events, vc), generator=g) ** 3).to(cuda)
    ids = torch.randint(0, n_det, (n_events,), generator=g, dtype=torch.int32).to(cuda)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    _lib.take_wait_timeout_count()
    tcd = tc.to(dtype)
    for grouped in (False, True):
        a = ops.sparse_weight_split(ids, tcd, A, tb, x, grouped=grouped, method="event")
        b = ops.sparse_weight_split(ids, tcd, A, tb, x, grouped=grouped)
        b2 = ops.sparse_weight_split(ids, tcd, A, tb, x, grouped=grouped)
        torch.cuda.synchronize()
        assert rel_l2(b.cpu(), a.cpu()) < TOL_W
        assert torch.equal(b, b2)
    assert _lib.take_wait_timeout_count() == 0


def test_grouped_bulk_scatter_wide_rings(cuda):
    """Two 8,208-theta rings on a stride-4 grid: fine tiles at the end of a ring, whose
    lateral taps wrap around to coarse theta 0, span more coarse voxels than one staged q
    segment and are scattered from global memory (the last one only partly filled), the
    other tiles from shared memory; all match the per-event kernel."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, synthetic
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    grid = synthetic.polar_grid(2, 8208, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    vc = p.coarse_pixel_num
    g = torch.Generator().manual_seed(7)
    n_det, n = 300, 1500
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(cuda).to(torch.bfloat16)
    tc = (torch.rand((n, vc), generator=g) ** 3).to(cuda).to(torch.bfloat16)
    ids = torch.randint(0, n_det, (n,), generator=g, dtype=torch.int32).to(cuda)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    _lib.take_wait_timeout_count()
    for grouped in (False, True):
        a = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped, method="event")
        b = ops.sparse_weight_split(ids, tc, A, tb, x, grouped=grouped)
        torch.cuda.synchronize()
        assert rel_l2(b.cpu(), a.cpu()) < TOL_W
    assert _lib.take_wait_timeout_count() == 0


def test_plan_groups_ahead_of_the_weight_call(cuda):
    """A grouping built ahead (ops.plan_groups) is the one the weight call then uses, and the
    weight equals the one computed with a fresh id tensor."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import ops, synthetic

    grid = synthetic.polar_grid(16, 96, 30.0)
    p = cso.build_compton_sparse_projector(grid.coor, 4, 1, rotate_num=1)
    tb = cso.tables(p, cuda)
    g = torch.Generator().manual_seed(5)
    n_det, n = 64, 900
    A = (torch.rand((n_det, grid.n_vox), generator=g) + 0.05).to(cuda).to(torch.bfloat16)
    tc = (torch.rand((n, p.coarse_pixel_num), generator=g) ** 3).to(cuda).to(torch.bfloat16)
    ids = torch.randint(0, n_det, (n,), generator=g, dtype=torch.int32).to(cuda)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.2).to(cuda)
    plan = ops.plan_groups(ids, n_det)
    w = ops.sparse_weight_split(ids, tc, A, tb, x)
    assert ids._jscc_group_plan[1] is plan
    w_fresh = ops.sparse_weight_split(ids.clone(), tc, A, tb, x)
    assert torch.equal(w, w_fresh)
    with pytest.raises(ValueError):
        ops.plan_groups(ids.long(), n_det)


def test_simple_model_rows_and_fused_weight(cuda):
    """The simple kernel (JSCC_CONE_SIMPLE: exp(-(beta - theta)^2 / 2 sigma_E^2) / d01^2 on the
    strict records): materialised rows against the float32 oracle restatement (per row,
    relative to the row maximum), and the fused on-the-fly weight against the stored rows'."""
    from jscc_recon_spect_cylinder_gb300 import _lib, ops
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop

    grid, det, sysmat, L, args = _cone_problem(cuda, n_events=1500)
    A, coor = sysmat.to(cuda), grid.coor.to(cuda)
    ev = pls.get_compton_event_params(A, det.to(cuda), coor, torch.from_numpy(L).to(cuda), *args,
                                      model=_lib.CONE_SIMPLE, theta_fp64=False, window_sigmas=0.0)
    assert len(ev) > 100
    tc, t = ops.compton_cone_rows(ev.records, ev.row_id, coor, model=_lib.CONE_SIMPLE, eff=A)
    ids = ev.list_index.cpu().numpy()
    cp1, cp2 = L[ids, 0].astype(np.int64), L[ids, 2].astype(np.int64)
    d = det.numpy()
    ref = oc.cone_rows_simple(d[cp1 - 1], d[cp2 - 1], L[ids, 1], grid.coor.numpy(), args[2], args[3],
                              dtype=np.float32)
    # without sigma_pos the Gaussian is only sigma_E wide, so an ulp of cos(beta) (amplified by
    # acos) moves t further than in the strict model: float32 and float64 evaluations of this
    # formula differ by up to 3e-4 per row on these events, two float32 ones by ~1e-4
    _rows_close(tc.cpu(), ref, 3e-4)
    x = torch.rand((grid.n_vox, 1), generator=torch.Generator().manual_seed(3)).to(cuda) + 0.5
    w_fused = ops.compton_weight(ev.records, ev.row_id, coor, x, model=_lib.CONE_SIMPLE, eff=A)
    w_stored = rop.get_weight_compton(t, x)
    assert rel_l2(w_fused.cpu(), w_stored.cpu()) < TOL_W
