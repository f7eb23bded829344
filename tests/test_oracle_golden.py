"""The CPU oracle against outputs of the reference's own functions (tests/golden)."""
from __future__ import annotations

import numpy as np

from conftest import rel_l2
from oracle import osem_sc


def _sc_inputs(g):
    S = int(g["n_subsets"])
    perm = g["perm"]
    bounds = osem_sc.split_even_bounds(perm.size, S)
    ids = [perm[a:b] for a, b in bounds]
    A_l = [[g["A0"][i], g["A1"][i]] for i in ids]
    y_l = [[g["y0"][i], g["y1"][i]] for i in ids]
    return A_l, y_l, [g["rot0"], g["rot1"]], [g["inv0"], g["inv1"]]


def test_split_even_matches_reference(golden):
    g = golden("sc_osem")
    for (n, k), sizes in zip(g["split_cases"], g["split_sizes"]):
        got = [b - a for a, b in osem_sc.split_even_bounds(int(n), int(k))]
        assert got == [int(s) for s in sizes[:k]]


def test_osem_bin_mode_matches_reference(golden):
    g = golden("sc_osem")
    A_l, y_l, rot, inv = _sc_inputs(g)
    R = rot[0].shape[1]
    img = np.ones((g["s"].shape[0], 1))
    for it, key in enumerate(("img_iter1", "img_iter2")):
        img32 = osem_sc.osem_bin_mode(A_l, y_l, rot, inv, img if it == 0 else img32, g["s"], R, dtype=np.float32)
        assert rel_l2(img32, g[key]) < 2e-6
    img64 = np.ones((g["s"].shape[0], 1))
    for _ in range(2):
        img64 = osem_sc.osem_bin_mode(A_l, y_l, rot, inv, img64, g["s"], R)
    assert rel_l2(img64, g["img_iter2"]) < 1e-5


def test_get_weight_single_matches_reference(golden):
    g = golden("sc_osem")
    x = np.ones((g["A0"].shape[1], 1))
    assert rel_l2(osem_sc.get_weight_single(g["A0"], g["y0"][:, :1], x), g["w_single"]) < 1e-6
    assert rel_l2(osem_sc.get_weight_single(g["A0"], g["y0"][:, :1], x, floor=1e-12), g["w_single_local"]) < 1e-6


def test_local_bin_mode_matches_reference(golden):
    g = golden("sc_osem")
    S = int(g["n_subsets"])
    img = np.ones((g["A0"].shape[1], 1))
    for perm in g["local_perms"]:
        ids = [perm[a:b] for a, b in osem_sc.chunk_bounds(perm.size, S)]
        img = osem_sc.osem_bin_mode([[g["A0"][i]] for i in ids], [[g["y0"][i]] for i in ids], [g["rot0"]],
                                    [g["inv0"]], img, g["s0"], g["rot0"].shape[1], floor=1e-12)
    assert rel_l2(img, g["local_img_iter2"]) < 1e-5


def _dense_t_list(g):
    S, D = int(g["n_subsets"]), int(g["n_divide"])
    R = g["rot"].shape[1]
    t_list = [[[[None] for _ in range(D)] for _ in range(R)] for _ in range(S)]
    for i in range(R):
        for j, (a, b) in enumerate(osem_sc.split_even_bounds(g["t"].shape[1], S)):
            ts = g["t"][i][a:b]
            for k, (c, d) in enumerate(osem_sc.split_even_bounds(ts.shape[0], D)):
                t_list[j][i][k][0] = ts[c:d]
    return t_list


def test_dense_list_and_joint_match_reference(golden):
    g = golden("dense_compton")
    R = g["rot"].shape[1]
    V = g["s"].shape[0]
    t_list = _dense_t_list(g)
    img = osem_sc.osem_list_mode(t_list, [g["rot"]], [g["inv"]], np.ones((V, 1)), g["s_d"], R)
    assert rel_l2(img, g["img_list"]) < 1e-5
    S = int(g["n_subsets"])
    ids = [np.arange(a, b) for a, b in osem_sc.split_even_bounds(g["A"].shape[0], S)]
    img = osem_sc.osem_joint_mode([[g["A"][i]] for i in ids], [[g["y"][i]] for i in ids], t_list, [g["rot"]],
                                  [g["inv"]], np.ones((V, 1)), 0.5 * g["s"] + 1.5 * g["s_d"], 0.5, R)
    assert rel_l2(img, g["img_joint"]) < 1e-5
    w = osem_sc.get_weight_compton(g["t"][0], np.ones((V, 1)))
    assert rel_l2(w, g["w_compton"]) < 1e-6


def test_safe_em_update_matches_reference(golden):
    g = golden("dense_compton")
    out = osem_sc.safe_em_update(g["safe_img"], g["safe_w"], g["safe_s"])
    np.testing.assert_allclose(out, g["safe_out"], rtol=1e-7, atol=0)


# ----------------------------------------------------------------------------- Compton builders
from oracle import compton as oc  # noqa: E402
from oracle import sparse as osp  # noqa: E402


def test_smearing_replays_reference(golden):
    g = golden("compton_builders")
    for tag in ("planar", "cyl"):
        a = g[f"{tag}_args"]
        e0, res = float(a[2]), float(a[3])
        L = g[f"{tag}_list"]
        e1 = oc.smear_energies(L[:, 1], g[f"{tag}_noise1"], e0, res)
        e2 = oc.smear_energies(L[:, 3], g[f"{tag}_noise2"], e0, res)
        np.testing.assert_allclose(e1, g[f"{tag}_smeared"][:, 1], rtol=2.5e-7, atol=0)
        np.testing.assert_allclose(e2, g[f"{tag}_smeared"][:, 3], rtol=2.5e-7, atol=0)


def _rows_close(a, b, rtol):
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-30)
    err = np.abs(a - b) / scale
    assert err.max() < rtol, err.max()


def test_strict_builder_matches_reference(golden):
    g = golden("compton_builders")
    for tag in ("planar", "cyl"):
        a = g[f"{tag}_args"]
        dr1, dr2, e0, res, tmax, tmin, tsum = [float(v) for v in a]
        for dtype, tol in ((np.float32, 2e-5), (np.float64, 2e-4)):
            t, tc, ts, kept = oc.strict_builder(g[f"{tag}_sysmat"], g[f"{tag}_det"], g["coor"], g[f"{tag}_smeared"],
                                                dr1, dr2, e0, res, tmax, tmin, tsum, dtype=dtype)
            _rows_close(t, g[f"{tag}_t"], tol)
            _rows_close(tc, g[f"{tag}_tc"], tol)
            _rows_close(ts, g[f"{tag}_ts"], 1e-6)


def test_legacy_builder_matches_reference(golden):
    g = golden("compton_builders")
    for tag in ("planar", "cyl"):
        a = g[f"{tag}_args"]
        dr, e0, res, tmax, tmin, tsum = 1.0 + float(a[0]), float(a[2]), float(a[3]), float(a[4]), float(a[5]), \
            float(a[6])
        t, tc, ts, _ = oc.legacy_builder(g[f"{tag}_sysmat"], g[f"{tag}_det"], g["coor"], g[f"{tag}_legacy_smeared"],
                                         dr, dr, e0, res, tmax, tmin, tsum, dtype=np.float32)
        # the legacy sigma formulas (atan, 1/sin theta derivatives, no clamps) amplify
        # float32 rounding more than the strict ones
        _rows_close(t, g[f"{tag}_legacy_t"], 1e-4)
        _rows_close(tc, g[f"{tag}_legacy_tc"], 1e-4)


# ----------------------------------------------------------------------------- sparse projector
def _dense_from(g, name):
    shape = tuple(g[f"r10_{name}_shape"])
    m = np.zeros(shape, np.float32)
    i = g[f"r10_{name}_idx"]
    m[i[0], i[1]] = g[f"r10_{name}_val"]
    return m


def test_projector_matches_reference_on_shipped_geometry(golden):
    g = golden("sparse_ops")
    p = osp.build_projector(g["r10_coor_full"], theta_stride=2, z_stride=2, rotate_num=10)
    assert tuple(p.ring_strides) == tuple(g["r10_ring_strides"])
    assert [p.fine_layer_num, p.fine_z_num, p.coarse_layer_num, p.coarse_z_num] == list(g["r10_dims"])
    for name in ("layer_reduce", "layer_expand", "z_reduce", "z_expand"):
        np.testing.assert_array_equal(getattr(p, name), _dense_from(g, name))
    np.testing.assert_allclose(p.coor_coarse, g["r10_coor_coarse"], rtol=0, atol=2e-5)
    np.testing.assert_allclose(osp.upsample_rows(g["r10_rows_c"], p), g["r10_up"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(osp.adjoint_rows(g["r10_rows_f"], p), g["r10_adj"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(osp.reduce_rows(g["r10_rows_f"], p), g["r10_red"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(osp.reduce_image(g["r10_img_f"], p), g["r10_img_red"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(osp.upsample_weight_image(g["r10_img_c"], p), g["r10_img_up"], rtol=1e-5, atol=1e-6)


def test_upsample_adjoint_pair_is_exact_in_fp64(golden):
    g = golden("sparse_ops")
    p = osp.build_projector(g["r10_coor_full"], theta_stride=2, z_stride=2, rotate_num=10)
    rng = np.random.default_rng(0)
    c = rng.random((2, p.coarse_pixel_num))
    f = rng.random((2, p.fine_pixel_num))
    lhs = np.sum(osp.upsample_rows(c, p) * f)
    rhs = np.sum(c * osp.adjoint_rows(f, p))
    assert abs(lhs - rhs) / abs(lhs) < 1e-13


def test_ring_stride_reduction_and_small_projector(golden):
    g = golden("sparse_ops")
    p = osp.build_projector(g["s_coor"], theta_stride=4, z_stride=2, rotate_num=4)
    assert tuple(p.ring_strides) == tuple(g["s_ring_strides"]) == (3,) * 6
    np.testing.assert_array_equal(p.layer_expand, g["s_layer_expand"])
    np.testing.assert_array_equal(p.z_expand, g["s_z_expand"])
    np.testing.assert_array_equal(p.layer_reduce, g["s_layer_reduce"])
    np.testing.assert_array_equal(p.z_reduce, g["s_z_reduce"])


def test_sparse_builder_and_weights_match_reference(golden):
    g = golden("sparse_ops")
    p = osp.build_projector(g["s_coor"], theta_stride=4, z_stride=2, rotate_num=4)
    p.coor_coarse = g["s_coor_coarse"]  # use the reference's float32 coarse coordinates
    a = [float(v) for v in g["s_args"]]
    rows, _ = osp.sparse_builder(g["s_sysmat"], g["s_det"], p, g["s_smeared"], *a, dtype=np.float64)
    ref = g["s_event_rows"]
    np.testing.assert_array_equal(rows[:, 0], ref[:, 0])
    _rows_close(rows[:, 1:], ref[:, 1:], 2e-4)
    t, valid = osp.materialize(ref, g["s_sysmat"], p)
    np.testing.assert_array_equal(valid, g["s_valid"])
    _rows_close(t, g["s_t_fine"], 1e-5)
    w_m = osp.weight_materialize(ref, g["s_sysmat"], g["s_x"], p)
    w_g = osp.weight_grouped(ref, g["s_sysmat"], g["s_x"], p)
    assert rel_l2(w_m, g["s_w_mat"]) < 1e-5
    assert rel_l2(w_g, g["s_w_grouped"]) < 1e-5
    # grouped and materialise forms agree (row-scale invariance of the list-mode weight)
    assert rel_l2(w_g, w_m) < 1e-5


def test_sparse_restatement_matches_dense_operators(golden):
    g = golden("sparse_ops")
    p = osp.build_projector(g["s_coor"], theta_stride=4, z_stride=2, rotate_num=4)
    U = osp.upsample_matrix_csr(p)
    rows = g["s_event_rows"]
    np.testing.assert_allclose((U @ rows[:, 1:].astype(np.float64).T).T, osp.upsample_rows(rows[:, 1:], p),
                               rtol=1e-12, atol=1e-15)
    w = osp.weight_materialize_csr(rows, g["s_sysmat"], g["s_x"], U)
    assert rel_l2(w, g["s_w_mat"]) < 1e-5


def test_sensitivity_builders_match_reference(golden):
    """Compton d (build_sparse_sensi_d_local, summed over two rotation blocks) and the SC
    sensitivity (compute_sensitivity_local over the shipped 10-view tables) against the
    reference's own outputs; the rescale of build_sparse_sensi_d on top of d."""
    from oracle import osem_sc

    g = golden("sensitivity")
    sp = golden("sparse_ops")
    p = osp.build_projector(sp["s_coor"], theta_stride=4, z_stride=2, rotate_num=4)
    rows, half = g["d_rows"], int(g["d_half"])
    d = osp.sensitivity_d(rows[:half], sp["s_sysmat"], p) + osp.sensitivity_d(rows[half:], sp["s_sysmat"], p)
    assert rel_l2(d, g["d_local"]) < 1e-6
    A = g["sc_codes"].astype(np.float32) * np.float32(2.0 ** -18)
    s = osem_sc.sc_sensitivity(A, sp["r10_rotmat_inv"], 10)
    assert rel_l2(s, g["sc_s"]) < 1e-6
    r = osp.sensitivity_d_rescale(d, s, 1000, 250)
    np.testing.assert_allclose(r.sum(), s.sum() * 250 / 1000, rtol=1e-12)
    assert np.array_equal(osp.sensitivity_d_rescale(np.zeros_like(d), s, 1, 1), np.zeros_like(d))


def test_simple_cone_oracle_is_the_strict_kernel_without_sigma_pos():
    """The simple restatement against the golden-pinned strict one: with zero position
    variance the strict kernel is exp(-(beta - theta)^2 / 2 sigma_E^2) (kn - sin^2 beta), so
    strict = simple * d01^2 * (kn - sin^2 beta) (float64, relative to each row's maximum; the
    strict kernel's floor of sigma_pos^2 at 1e-12 is the only difference, ~1e-8 here)."""
    from oracle import compton as oc

    rng = np.random.default_rng(8)
    n, e0 = 40, 0.511
    pos1 = rng.uniform(-120, 120, (n, 3))
    pos2 = rng.uniform(-150, 150, (n, 3))
    e1 = rng.uniform(0.08, 0.3, n)
    coor = rng.uniform(-40, 40, (300, 3))
    res = 0.1
    zero = np.zeros((n, 3))
    strict = oc.cone_rows_strict(pos1, pos2, e1, zero, zero, coor, e0, res)
    simple = oc.cone_rows_simple(pos1, pos2, e1, coor, e0, res)
    v01 = pos1[:, None, :] - coor[None, :, :]
    v12 = (pos2 - pos1)[:, None, :]
    d01 = np.linalg.norm(v01, axis=-1)
    bcos = (v01 * v12).sum(-1) / np.maximum(d01 * np.linalg.norm(v12, axis=-1), 1e-7)
    c = np.clip(bcos, -1 + 1e-7, 1 - 1e-7)
    kn = e0 / (e0 - e1) + (e0 - e1) / e0
    expect = simple * d01 ** 2 * (kn[:, None] - (1 - c) * (1 + c))
    scale = np.maximum(np.abs(strict).max(axis=1, keepdims=True), 1e-300)  # rows that underflow entirely
    assert np.max(np.abs(strict - expect) / scale) < 1e-6
