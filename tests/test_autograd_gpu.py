"""Differentiable projectors (autograd.SCProject / ComptonProject): the backward is the
exact adjoint of the forward (dot-product identity), the Poisson log-likelihood gradient
equals the reference's OSEM backprojection minus the sensitivity (recon_osem_plane.py:28-42),
and central finite differences agree (float32 projections, float64 sums: 1e-3)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _sc(cuda, n_bins=200, n_r=8, n_theta=24, R=4, seed=0):
    from jscc_recon_spect_cylinder_gb300 import synthetic

    g = torch.Generator().manual_seed(seed)
    V = n_r * n_theta
    A = (torch.rand((n_bins, V), generator=g) + 0.05).to(cuda)
    rot, inv = synthetic.cyclic_rotation_tables(n_r, n_theta, R)
    y = torch.poisson(torch.rand((n_bins, R), generator=g) * 50 + 5, generator=g).to(cuda)
    x = (torch.rand((V, 1), generator=g) + 0.2).to(cuda)
    return A, rot.to(cuda), inv.to(cuda), y, x


def _cone(cuda, n_events=1500, seed=4):
    from jscc_recon_spect_cylinder_gb300 import process_list_plane_strict as pls
    from jscc_recon_spect_cylinder_gb300 import synthetic

    grid = synthetic.polar_grid(12, 48, 40.0)
    scat = synthetic.cylinder_pixels(120.0, 32, 4, 3.0)
    absb = synthetic.cylinder_pixels(150.0, 32, 4, 3.0)
    det = torch.cat((scat, absb)).float()
    g = torch.Generator().manual_seed(seed)
    sysmat = (torch.rand((det.size(0), grid.n_vox), generator=g) * 1e-3 + 1e-5).to(cuda)
    rng = np.random.default_rng(seed)
    e0 = 0.511
    cp1 = rng.integers(1, scat.size(0) + 1, n_events)
    cp2 = rng.integers(scat.size(0) + 1, det.size(0) + 1, n_events)
    e1 = rng.uniform(0.08, 0.3, n_events)
    L = torch.from_numpy(np.stack((cp1, e1, cp2, e0 - e1), axis=1).astype(np.float32)).to(cuda)
    res = 0.1 * (0.662 / e0) ** 0.5
    args = (0.8, 0.8, e0, res, 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001, 0.05, e0 - 0.06)
    coor = grid.coor.to(cuda).float()
    ev = pls.get_compton_event_params(sysmat, det.to(cuda), coor, L, *args, window_sigmas=0.0)
    x = (torch.rand((grid.n_vox, 1), generator=g) + 0.5).to(cuda)
    return ev, coor, sysmat, x


def test_sc_adjoint_dot_product(cuda):
    from jscc_recon_spect_cylinder_gb300 import autograd as ag

    A, rot, inv, y, x = _sc(cuda)
    f = ag.sc_project(x, A, rot, inv, 4)
    g = torch.rand_like(f)
    xg = x.clone().requires_grad_(True)
    (ag.sc_project(xg, A, rot, inv, 4) * g).sum().backward()
    lhs = float((f.double() * g.double()).sum())
    rhs = float((x.double() * xg.grad.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-6
    # forward against torch (float64) on the rotated images
    ref = torch.stack([A.double() @ x.double().reshape(-1)[rot[:, r] - 1] for r in range(4)], dim=1)
    assert rel_l2(f.cpu(), ref.cpu()) < 1e-6


def test_sc_likelihood_gradient_is_osem_weight_minus_sensitivity(cuda):
    from jscc_recon_spect_cylinder_gb300 import autograd as ag
    from jscc_recon_spect_cylinder_gb300 import ops

    A, rot, inv, y, x = _sc(cuda)
    xg = x.clone().requires_grad_(True)
    ag.poisson_log_likelihood(xg, sc=(A, y, rot, inv)).backward()
    w = ops.sc_weight(A, y, x, rotmat=rot, rotmat_inv=inv)  # sum_r rotinv_r A^T (y_r / A rot_r x)
    s = ops.sc_sensitivity(A, inv) * 4                      # sum_r rotinv_r A^T 1
    assert rel_l2(xg.grad.cpu(), (w - s).cpu()) < 1e-5


def test_compton_adjoint_and_gradient(cuda):
    from jscc_recon_spect_cylinder_gb300 import autograd as ag
    from jscc_recon_spect_cylinder_gb300 import ops

    ev, coor, sysmat, x = _cone(cuda)
    assert len(ev) > 100
    f = ag.compton_project(x, ev, coor, sysmat)
    g = torch.rand_like(f)
    xg = x.clone().requires_grad_(True)
    (ag.compton_project(xg, ev, coor, sysmat) * g).sum().backward()
    lhs = float((f.double() * g.double()).sum())
    rhs = float((x.double() * xg.grad.double()).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-6
    # list-mode likelihood gradient = T^T (1 / T x) - s_C (the fused OSEM weight)
    s_c = ops.compton_backproject(ev.records, ev.row_id, coor, torch.ones_like(f), model=ev.model, eff=sysmat)
    assert float(f.min()) > 0  # every event sees the image: 1/f is finite for all of them
    xg = x.clone().requires_grad_(True)
    ag.poisson_log_likelihood(xg, compton=(ev, coor, sysmat, s_c)).backward()
    w = ops.compton_weight(ev.records, ev.row_id, coor, x, model=ev.model, eff=sysmat)
    assert rel_l2(xg.grad.cpu(), (w - s_c).cpu()) < 1e-5


def test_joint_likelihood_finite_differences(cuda):
    """Central differences of L(x) along random directions against <grad L, d>. The
    projections are float32 and L is summed in float64, so they agree to 1e-3."""
    from jscc_recon_spect_cylinder_gb300 import autograd as ag

    A, rot, inv, y, x = _sc(cuda, n_r=12, n_theta=48)
    ev, coor, sysmat, _ = _cone(cuda)
    s_c = torch.rand_like(x) * 0.01
    sc, cp = (A, y, rot, inv), (ev, coor, sysmat, s_c)
    xg = x.clone().requires_grad_(True)
    ag.poisson_log_likelihood(xg, sc=sc, compton=cp).backward()
    gen = torch.Generator().manual_seed(9)
    for _ in range(3):
        d = (torch.rand(x.shape, generator=gen) - 0.5).to(cuda)
        eps = 1e-2
        lp = float(ag.poisson_log_likelihood(x + eps * d, sc=sc, compton=cp))
        lm = float(ag.poisson_log_likelihood(x - eps * d, sc=sc, compton=cp))
        fd = (lp - lm) / (2 * eps)
        an = float((xg.grad * d).sum())
        assert abs(fd - an) / max(abs(an), 1e-12) < 1e-3, (fd, an)
