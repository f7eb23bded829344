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
