"""MAP objective oracle and neighbour tables (CPU): the float64 gradients of the prior and of
the joint log-posterior agree with float64 central differences, and the polar neighbour
tables are the 4- (default) or 8-neighbourhood on uniform grids and symmetric on rings of
different lengths and on several z layers."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from oracle import map as om


def _table(coor, **kw):
    from jscc_recon_spect_cylinder_gb300 import prior

    return prior.polar_neighbours(coor, **kw)


def _grid(n_r, n_theta):
    from jscc_recon_spect_cylinder_gb300 import synthetic

    return synthetic.polar_grid(n_r, n_theta, 20.0).coor


def _variable_rings(lengths=(6, 12, 18, 24), n_z=2, pitch=2.0):
    pts = []
    for z in range(n_z):
        for r, L in enumerate(lengths):
            th = 2 * math.pi * (np.arange(L) + 0.5 * (r % 2)) / L
            rr = (r + 0.5) * 3.0
            pts.append(np.stack((rr * np.cos(th), rr * np.sin(th), np.full(L, z * pitch)), axis=1))
    return torch.from_numpy(np.concatenate(pts).astype(np.float32))


def _directed(tb):
    nbr, w = tb.nbr.numpy(), tb.weight.numpy()
    out = {}
    for k in range(nbr.shape[0]):
        for j in range(nbr.shape[1]):
            if nbr[k, j] >= 0:
                assert (j, int(nbr[k, j])) not in out, "duplicate edge"
                out[(j, int(nbr[k, j]))] = float(w[k, j])
            else:
                assert w[k, j] == 0
    return out


@pytest.mark.parametrize("diagonal", [False, True])
def test_uniform_grid_neighbourhoods(diagonal):
    """Default: ring +-1 angle and the same angle in the adjacent rings (4-neighbourhood);
    with diagonals, the 8-neighbourhood with weights 1 and 1/sqrt(2)."""
    n_r, n_t = 5, 8
    e = _directed(_table(_grid(n_r, n_t), diagonal=diagonal))
    steps = ((0, 1), (0, -1), (1, 0), (-1, 0))
    if diagonal:
        steps += ((1, 1), (1, -1), (-1, 1), (-1, -1))
    want = {}
    for r in range(n_r):
        for t in range(n_t):
            j = r * n_t + t
            for dr, dt in steps:
                if 0 <= r + dr < n_r:
                    want[(j, (r + dr) * n_t + (t + dt) % n_t)] = 1.0 if dr == 0 or dt == 0 else 1 / math.sqrt(2)
    assert set(e) == set(want)
    for key, w in want.items():
        assert abs(e[key] - w) < 1e-7


def test_variable_rings_and_layers_are_symmetric():
    coor = _variable_rings()
    for w, diag in (("index", False), ("index", True), ("distance", True)):
        e = _directed(_table(coor, weights=w, diagonal=diag))
        for (j, k), wt in e.items():
            assert j != k
            assert e.get((k, j)) == wt
    e = _directed(_table(coor))
    n_layer = 6 + 12 + 18 + 24
    # z faces: every voxel of layer 0 sees the same slot of layer 1
    for j in range(n_layer):
        assert e[(j, j + n_layer)] == 1.0
    # every voxel has its two in-ring neighbours, the nearest slot of each adjacent ring and
    # its z face: at least 4 (innermost / outermost ring: one adjacent ring)
    for j in range(n_layer):
        assert sum(1 for (a, _) in e if a == j) >= 4


def test_rdp_gradient_matches_central_differences():
    coor = _grid(6, 12)
    tb = _table(coor)
    rng = np.random.default_rng(1)
    x = rng.uniform(0.2, 2.0, coor.size(0))
    x[5] = x[6]  # a zero difference
    for gamma in (0.0, 2.0):
        _, g = om.rdp(x, tb.nbr.numpy(), tb.weight.numpy(), gamma)
        h = 1e-6
        fd = np.empty_like(x)
        for j in range(x.size):
            e = np.zeros_like(x)
            e[j] = h
            fd[j] = (om.rdp(x + e, tb.nbr.numpy(), tb.weight.numpy(), gamma)[0]
                     - om.rdp(x - e, tb.nbr.numpy(), tb.weight.numpy(), gamma)[0]) / (2 * h)
        assert np.max(np.abs(fd - g)) < 1e-6 * max(1.0, np.max(np.abs(g)))


def test_map_objective_gradient_matches_central_differences():
    from jscc_recon_spect_cylinder_gb300 import synthetic

    n_r, n_t, R = 5, 12, 3
    coor = _grid(n_r, n_t)
    V = coor.size(0)
    rot, _ = synthetic.cyclic_rotation_tables(n_r, n_t, R)
    rng = np.random.default_rng(2)
    A = rng.uniform(0.05, 1.0, (30, V))
    y = rng.poisson(20.0, (30, R)).astype(np.float64)
    T = rng.uniform(0.0, 1.0, (40, V)) ** 3
    s_c = rng.uniform(0.0, 0.5, V)
    tb = _table(coor)
    prior = (tb.nbr.numpy(), tb.weight.numpy(), 0.3, 2.0, 1e-9)
    z = np.log(rng.uniform(0.3, 3.0, V))
    _, g = om.map_objective(z, sc=(A, y, rot.numpy()), compton=(T, s_c), prior=prior)
    for _ in range(3):
        d = rng.standard_normal(V)
        h = 1e-5
        fp = om.map_objective(z + h * d, sc=(A, y, rot.numpy()), compton=(T, s_c), prior=prior)[0]
        fm = om.map_objective(z - h * d, sc=(A, y, rot.numpy()), compton=(T, s_c), prior=prior)[0]
        fd = (fp - fm) / (2 * h)
        an = float(g @ d)
        assert abs(fd - an) < 1e-7 * max(1.0, abs(an)), (fd, an)


def test_sc_likelihood_gradient_is_the_osem_backprojection():
    """dL_SC/dx = sum_r rotinv_r(A^T (y_r / f_r)) - sum_r rotinv_r(A^T 1): the reference's
    get_weight_single backprojection minus R times its sensitivity (recon_osem_plane.py:28-30,
    51; main_local_cntstat.py:140-146 averages over the R views)."""
    from jscc_recon_spect_cylinder_gb300 import synthetic
    from oracle import osem_sc

    n_r, n_t, R = 4, 12, 4
    rot, inv = synthetic.cyclic_rotation_tables(n_r, n_t, R)
    rng = np.random.default_rng(3)
    V = n_r * n_t
    A = rng.uniform(0.05, 1.0, (25, V))
    y = rng.poisson(10.0, (25, R)).astype(np.float64)
    x = rng.uniform(0.3, 2.0, V)
    _, g = om.sc_log_likelihood(x, A, y, rot.numpy())
    w = np.zeros(V)
    for r in range(R):
        xr = x[rot.numpy()[:, r] - 1][:, None]
        wr = osem_sc.get_weight_single(A, y[:, r:r + 1], xr).ravel()
        w += wr[inv.numpy()[:, r] - 1]
    s = osem_sc.sc_sensitivity(A, inv.numpy(), R).ravel() * R  # the reference's s is the mean over views
    assert np.allclose(g, w - s, rtol=1e-10, atol=1e-10)


def test_adam_restatement_matches_torch():
    rng = np.random.default_rng(4)
    target = rng.standard_normal(7)

    def f(z):
        return float(np.sum((z - target) ** 4)), 4 * (z - target) ** 3

    z0 = np.zeros(7)
    z, _ = om.adam(f, z0, 0.05, 25)
    zt = torch.zeros(7, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([zt], lr=0.05)
    tt = torch.from_numpy(target)
    for _ in range(25):
        opt.zero_grad()
        ((zt - tt) ** 4).sum().backward()
        opt.step()
    assert np.allclose(z, zt.detach().numpy(), rtol=1e-12, atol=1e-12)


def test_neighbours_on_the_shipped_geometry(golden):
    """The reference's shipped r10 polar grid (20 planes x 25 rings of 10-80 voxels): the
    table is symmetric without duplicates or self edges, every voxel has its two in-ring
    neighbours and its z faces and at least one neighbour in an adjacent ring, and the prior's
    value over the table equals the direct sum over its undirected edges."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    coor = torch.from_numpy(golden("sparse_ops")["r10_coor_full"])
    lay = cso._infer_polar_layout(coor)
    n_layer, n_z = int(lay["fine_layer_num"]), int(lay["fine_z_num"])
    lengths = [int(v) for v in lay["ring_lengths"]]
    tb = _table(coor)
    nbr = tb.nbr.numpy()
    V = coor.size(0)
    pairs = set()
    for k in range(nbr.shape[0]):
        for j in np.nonzero(nbr[k] >= 0)[0]:
            pairs.add((int(j), int(nbr[k, j])))
    assert len(pairs) == int((nbr >= 0).sum())  # no duplicates
    assert all((b, a) in pairs for a, b in pairs)
    assert all(a != b for a, b in pairs)
    starts = np.concatenate(([0], np.cumsum(lengths)[:-1]))
    for z in (0, n_z // 2, n_z - 1):
        for r, L in enumerate(lengths):
            for t in (0, L // 2, L - 1):
                j = z * n_layer + starts[r] + t
                mine = {b for a, b in pairs if a == j}
                assert {z * n_layer + starts[r] + (t + 1) % L, z * n_layer + starts[r] + (t - 1) % L} <= mine
                if z > 0:
                    assert j - n_layer in mine
                if z + 1 < n_z:
                    assert j + n_layer in mine
                in_plane = {b - z * n_layer for b in mine if z * n_layer <= b < (z + 1) * n_layer}
                assert any(not starts[r] <= b < starts[r] + L for b in in_plane), (z, r, t)  # an adjacent ring
    x = np.random.default_rng(6).uniform(0.5, 2.0, V)
    value, _ = om.rdp(x, nbr, tb.weight.numpy(), 2.0)
    direct = sum(1.0 * (x[a] - x[b]) ** 2 / (x[a] + x[b] + 2.0 * abs(x[a] - x[b]) + 1e-9) for a, b in pairs if a < b)
    assert abs(value - direct) < 1e-9 * direct
