"""MAP reconstruction on the GPU: the relative-difference prior kernel against the float64
oracle, the log-posterior gradient (SC + Compton + prior through autograd) against the
float64 oracle and its finite differences on a 20 x 60 grid with 5k events, and the Adam
MAP loop against the oracle's Adam."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import compton as oc
from oracle import map as om

pytestmark = pytest.mark.gpu

N_R, N_T, R = 20, 60, 4


def _variable_rings(lengths=(6, 12, 18, 24, 30), n_z=3):
    pts = []
    for z in range(n_z):
        for r, L in enumerate(lengths):
            th = 2 * math.pi * (np.arange(L) + 0.5 * (r % 2)) / L
            rr = (r + 0.5) * 3.0
            pts.append(np.stack((rr * np.cos(th), rr * np.sin(th), np.full(L, 2.0 * z)), axis=1))
    return torch.from_numpy(np.concatenate(pts).astype(np.float32))


@pytest.mark.parametrize("grid", ["uniform", "rings"])
@pytest.mark.parametrize("gamma", [0.0, 2.0])
def test_rdp_kernel_matches_oracle(cuda, grid, gamma):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, prior, synthetic

    coor = synthetic.polar_grid(N_R, N_T, 50.0).coor if grid == "uniform" else _variable_rings()
    tb = prior.polar_neighbours(coor, weights="index" if grid == "uniform" else "distance",
                                diagonal=grid != "uniform")
    V = coor.size(0)
    rng = np.random.default_rng(5)
    x = rng.uniform(0.1, 3.0, V).astype(np.float32)
    x[:V // 7] = 1.0  # flat patches: zero differences
    beta = 0.37
    val, g = ops.rdp_prior(torch.from_numpy(x).to(cuda), tb.nbr.to(cuda), tb.weight.to(cuda), gamma=gamma, beta=beta)
    rv, rg = om.rdp(x, tb.nbr.numpy(), tb.weight.numpy(), gamma)
    assert abs(float(val) - beta * rv) <= 1e-5 * abs(beta * rv)
    # the value is reduced in a fixed order (no float atomics): repeated calls are bit-identical
    for _ in range(3):
        v_again, g_again = ops.rdp_prior(torch.from_numpy(x).to(cuda), tb.nbr.to(cuda), tb.weight.to(cuda),
                                         gamma=gamma, beta=beta)
        assert float(v_again) == float(val) and torch.equal(g_again, g)
    assert rel_l2(g.cpu(), beta * rg) < 1e-5
    # accumulate into an existing gradient, gradient only
    base = torch.rand((V, 1), device=cuda)
    acc = base.clone()
    v2, g2 = ops.rdp_prior(torch.from_numpy(x).to(cuda), tb.nbr.to(cuda), tb.weight.to(cuda), gamma=gamma, beta=beta,
                           want_value=False, grad_out=acc, accumulate=True)
    assert v2 is None and g2 is acc
    assert rel_l2((acc - base).cpu(), beta * rg) < 1e-5
    assert _lib.take_bad_index_count() == 0


def test_rdp_kernel_skips_and_counts_bad_indices(cuda):
    from jscc_recon_spect_cylinder_gb300 import _lib, ops, prior, synthetic

    coor = synthetic.polar_grid(6, 12, 10.0).coor
    tb = prior.polar_neighbours(coor)
    V = coor.size(0)
    nbr = tb.nbr.clone()
    # slot 0 of voxel 3 points past the end: the kernel skips it (and counts it)
    nbr[0, 3] = V + 5
    x = torch.rand(V, generator=torch.Generator().manual_seed(2)) + 0.5
    _lib.take_bad_index_count()
    val, g = ops.rdp_prior(x.to(cuda), nbr.to(cuda), tb.weight.to(cuda))
    torch.cuda.synchronize()
    assert _lib.take_bad_index_count() == 1
    nb = nbr.numpy().copy()
    nb[0, 3] = -1
    _, rg = om.rdp(x.numpy(), nb, tb.weight.numpy(), 2.0)
    # voxel 3 lost one directed term of its gradient, nothing else changed
    assert rel_l2(np.delete(g.cpu().numpy().ravel(), 3), np.delete(rg, 3)) < 1e-5


def _joint_problem(cuda, n_events=5000, seed=7):
    """Config-5 sub-problem: 20 x 60 polar grid (50 mm disk), SC channel of 256 pixels x 4
    views (rotation tables), 5k two-interaction events at 662 keV on scatter / absorber
    cylinders; the event records evaluate every pair (no window) with a float32 theta so the
    float32 oracle cone rows are the same function."""
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import synthetic

    prob = synthetic.sc_problem(n_r=N_R, n_theta=N_T, n_phi=256, views=R, flat=False, total_counts=2e5)
    coor = prob.grid.coor
    scat = synthetic.cylinder_pixels(120.0, 32, 4, 3.0)
    absb = synthetic.cylinder_pixels(150.0, 32, 4, 3.0)
    det = torch.cat((scat, absb)).float()
    g = torch.Generator().manual_seed(seed)
    eff = torch.rand((det.size(0), coor.size(0)), generator=g) * 1e-3 + 1e-5
    rng = np.random.default_rng(seed)
    e0 = 0.662
    cp1 = rng.integers(1, scat.size(0) + 1, n_events)
    cp2 = rng.integers(scat.size(0) + 1, det.size(0) + 1, n_events)
    e1 = rng.uniform(0.1, 0.4, n_events)
    L = np.stack((cp1, e1, cp2, e0 - e1), axis=1).astype(np.float32)
    res = 0.08 * (0.662 / e0) ** 0.5
    args = (0.8, 0.8, e0, res, 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001, 0.05, e0 - 0.06)
    ev = pls.get_compton_event_params(eff.to(cuda), det.to(cuda), coor.to(cuda), torch.from_numpy(L).to(cuda), *args,
                                      theta_fp64=False, window_sigmas=0.0)
    ids = ev.list_index.cpu().numpy()
    c1, c2 = L[ids, 0].astype(np.int64), L[ids, 2].astype(np.int64)
    d = det.numpy()
    s1, s2 = oc.pos_sigma_sq(d, args[0]), oc.pos_sigma_sq(d, args[1])
    rows = []
    for a in range(0, ids.size, 1000):  # float32 cone rows in event chunks (bounded host memory)
        sl = slice(a, a + 1000)
        rows.append(oc.cone_rows_strict(d[c1[sl] - 1], d[c2[sl] - 1], L[ids[sl], 1], s1[c1[sl] - 1], s2[c2[sl] - 1],
                                        coor.numpy(), e0, res, dtype=np.float32))
    T = np.concatenate(rows).astype(np.float64) * eff.numpy().astype(np.float64)[c1 - 1]
    return prob, ev, coor, eff, T


def test_map_gradient_matches_fp64_oracle_and_finite_differences(cuda):
    """Config-5 gradient check: Phi(z) = -L_SC(e^z) - L_C(e^z) + beta R(e^z), beta = 0.01,
    gamma = 2. The GPU gradient (forward/adjoint kernels + prior kernel through autograd)
    against the float64 oracle gradient, and against float64 central differences of the
    oracle objective along random directions."""
    from jscc_recon_spect_cylinder_gb300 import autograd as ag
    from jscc_recon_spect_cylinder_gb300 import ops, prior

    prob, ev, coor, eff, T = _joint_problem(cuda)
    assert len(ev) > 500  # of 5,000 listed: the energy, kinematic and row filters keep ~15 %
    V = coor.size(0)
    tb = prior.polar_neighbours(coor)
    A, y, rot, inv = (t.to(cuda) for t in (prob.sysmat, prob.proj, prob.rotmat, prob.rotmat_inv))
    s_c = ops.compton_backproject(ev.records, ev.row_id, coor.to(cuda), torch.ones(len(ev), device=cuda),
                                  model=ev.model, eff=eff.to(cuda))
    beta, gamma = 0.01, 2.0
    z0 = np.log(np.random.default_rng(8).uniform(0.3, 3.0, V))
    z = torch.from_numpy(z0).float().to(cuda).reshape(V, 1).requires_grad_(True)
    x = torch.exp(z)
    tbd = tb.to(cuda)
    obj = (-ag.poisson_log_likelihood(x, sc=(A, y, rot, inv), compton=(ev, coor.to(cuda), eff.to(cuda), s_c))
           + ag.rdp_prior(x, tbd, beta=beta, gamma=gamma))
    obj.backward()
    g_gpu = z.grad.double().cpu().numpy().ravel()

    zz = z.detach().double().cpu().numpy().ravel()  # the float32 z the GPU saw
    sc = (prob.sysmat.numpy(), prob.proj.numpy(), prob.rotmat.numpy())
    cp = (T, s_c.double().cpu().numpy())
    pr = (tb.nbr.numpy(), tb.weight.numpy(), beta, gamma, 1e-9)
    v64, g64 = om.map_objective(zz, sc=sc, compton=cp, prior=pr)
    val = float(obj.detach())
    assert abs(val - v64) <= 1e-5 * abs(v64), (val, v64)
    assert rel_l2(g_gpu, g64) < 1e-4
    rng = np.random.default_rng(9)
    for _ in range(3):
        dvec = rng.standard_normal(V)
        h = 1e-5
        fd = (om.map_objective(zz + h * dvec, sc=sc, compton=cp, prior=pr)[0]
              - om.map_objective(zz - h * dvec, sc=sc, compton=cp, prior=pr)[0]) / (2 * h)
        assert abs(float(g64 @ dvec) - fd) <= 1e-6 * abs(fd)        # the oracle is its own calculus
        assert abs(float(g_gpu @ dvec) - fd) <= 1e-4 * abs(fd), (float(g_gpu @ dvec), fd)


def test_map_reconstruct_tracks_oracle_adam(cuda):
    """20 Adam steps of map_reconstruct (lr 0.05 in log-intensity) against the oracle's
    float64 Adam on the same objective: the objective histories agree to 1e-4 and decrease."""
    from jscc_recon_spect_cylinder_gb300 import autograd as ag
    from jscc_recon_spect_cylinder_gb300 import ops, prior

    prob, ev, coor, eff, T = _joint_problem(cuda, n_events=2000)
    V = coor.size(0)
    tb = prior.polar_neighbours(coor)
    A, y, rot, inv = (t.to(cuda) for t in (prob.sysmat, prob.proj, prob.rotmat, prob.rotmat_inv))
    s_c = ops.compton_backproject(ev.records, ev.row_id, coor.to(cuda), torch.ones(len(ev), device=cuda),
                                  model=ev.model, eff=eff.to(cuda))
    x0 = torch.ones((V, 1), device=cuda)
    n, lr, beta = 20, 0.05, 0.01
    x, hist = ag.map_reconstruct(x0, sc=(A, y, rot, inv), compton=(ev, coor.to(cuda), eff.to(cuda), s_c),
                                 table=tb.to(cuda), beta=beta, gamma=2.0, n_steps=n, lr=lr)
    sc = (prob.sysmat.numpy(), prob.proj.numpy(), prob.rotmat.numpy())
    cp = (T, s_c.double().cpu().numpy())
    pr = (tb.nbr.numpy(), tb.weight.numpy(), beta, 2.0, 1e-9)
    z64, h64 = om.adam(lambda zz: om.map_objective(zz, sc=sc, compton=cp, prior=pr), np.zeros(V), lr, n)
    h = hist.numpy()
    assert np.all(np.isfinite(h))
    assert h[-1] < h[0]
    assert np.max(np.abs(h - h64) / np.abs(h64)) < 1e-4, (h, h64)
    assert rel_l2(x.cpu().numpy().ravel(), np.exp(z64)) < 1e-2


def test_fp64_gradient_matches_finite_differences(cuda):
    """With float64 images the projector halves and the prior run their FP64 forms
    (jscc_*_f64): the autograd gradient of Phi(z) = -L_SC(e^z) - L_C(e^z) + beta R(e^z) on the
    20 x 60 grid with 5k listed events matches FP64 central differences to 1e-6 along random
    directions, and the float32 kernels' gradient to 1e-3."""
    from jscc_recon_spect_cylinder_gb300 import autograd as ag
    from jscc_recon_spect_cylinder_gb300 import ops, prior

    prob, ev, coor, eff, _ = _joint_problem(cuda)
    V = coor.size(0)
    tb = prior.polar_neighbours(coor).to(cuda)
    A, y, rot, inv = (t.to(cuda) for t in (prob.sysmat, prob.proj, prob.rotmat, prob.rotmat_inv))
    cc, ec = coor.to(cuda), eff.to(cuda)

    def objective(z, dtype):
        s_c = ops.compton_backproject(ev.records, ev.row_id, cc, torch.ones(len(ev), dtype=dtype, device=cuda),
                                      model=ev.model, eff=ec)
        x = torch.exp(z)
        return (-ag.poisson_log_likelihood(x, sc=(A, y, rot, inv), compton=(ev, cc, ec, s_c.detach()))
                + ag.rdp_prior(x, tb, beta=0.01, gamma=2.0))

    z0 = torch.from_numpy(np.log(np.random.default_rng(8).uniform(0.3, 3.0, V))).reshape(V, 1)
    z = z0.to(cuda).double().requires_grad_(True)
    objective(z, torch.float64).backward()
    g = z.grad.detach()
    assert g.dtype == torch.float64
    z32 = z0.to(cuda).float().requires_grad_(True)
    objective(z32, torch.float32).backward()
    assert rel_l2(z32.grad.double().cpu(), g.cpu()) < 1e-3
    gen = torch.Generator().manual_seed(21)
    h = 1e-6
    with torch.no_grad():
        for _ in range(3):
            d = torch.randn((V, 1), generator=gen, dtype=torch.float64).to(cuda)
            fd = (float(objective(z.detach() + h * d, torch.float64))
                  - float(objective(z.detach() - h * d, torch.float64))) / (2 * h)
            an = float((g * d).sum())
            assert abs(fd - an) <= 1e-6 * abs(fd), (fd, an)
