"""The radially coarsened Compton projector (an extension: the reference's
build_compton_sparse_projector coarsens theta and z only, compton_sparse_ops.py:212-290),
host construction only (CPU). There is no reference behaviour for radial coarsening, so the
builder is pinned three ways: (1) it equals the oracle's independent numpy restatement entry
by entry; (2) with radial stride 1 its upsample and coarse coordinates equal the reference's
own projector (theta stride s, z stride 1), through the golden-pinned oracle; (3) the maps
interpolate: rows of the upsample sum to one, and a coarse image sampled from a function
linear in the ring index and constant in theta is reproduced exactly on the rings between the
first and last coarse centres."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import sparse as osp


def _grid(rings=16, theta=96, planes=1):
    from jscc_recon_spect_cylinder_gb300 import synthetic

    g = synthetic.polar_grid(rings, theta, 30.0)
    c = g.coor.numpy()
    if planes == 1:
        return c
    return np.concatenate([np.concatenate((c[:, :2], np.full((c.shape[0], 1), 2.0 * k, np.float32)), axis=1)
                           for k in range(planes)], axis=0)


@pytest.mark.parametrize("rings,theta,planes,rs,ts", [(16, 96, 1, 4, 4), (12, 48, 2, 2, 4), (100, 360, 1, 4, 4)])
def test_radial_builder_matches_oracle(rings, theta, planes, rs, ts):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    c = _grid(rings, theta, planes)
    p = cso.build_compton_sparse_projector_radial(torch.from_numpy(c), rs, ts)
    o = osp.build_radial_projector(c, rs, ts)
    for f in ("layer_reduce", "z_reduce", "layer_expand", "z_expand"):
        np.testing.assert_array_equal(getattr(p, f).numpy(), getattr(o, f))
    np.testing.assert_allclose(p.coor_coarse.numpy(), o.coor_coarse, atol=1e-4, rtol=0)
    assert (p.fine_pixel_num, p.coarse_pixel_num) == (o.fine_pixel_num, o.coarse_pixel_num)
    assert p.coarse_pixel_num == planes * (rings // rs) * (theta // ts)
    assert p.radial_stride == rs and p.ring_num == rings


def test_radial_stride_one_is_the_reference_projector():
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    c = _grid(12, 48, 2)
    o1 = osp.build_radial_projector(c, 1, 4)
    ref = osp.build_projector(c, theta_stride=4, z_stride=1)
    np.testing.assert_array_equal(osp.upsample_matrix_csr(o1).toarray(), osp.upsample_matrix_csr(ref).toarray())
    np.testing.assert_array_equal(o1.coor_coarse, ref.coor_coarse)
    p1 = cso.build_compton_sparse_projector_radial(torch.from_numpy(c), 1, 4)
    pr = cso.build_compton_sparse_projector(torch.from_numpy(c), theta_stride=4, z_stride=1)
    up1 = torch.kron(p1.z_expand, p1.layer_expand)
    upr = torch.kron(pr.z_expand, pr.layer_expand)
    assert torch.equal(up1, upr)


def test_radial_maps_interpolate():
    rings, theta, rs, ts = 16, 96, 4, 4
    o = osp.build_radial_projector(_grid(rings, theta), rs, ts)
    U = osp.upsample_matrix_csr(o)
    np.testing.assert_allclose(np.asarray(U.sum(axis=1)).ravel(), 1.0, atol=1e-6)
    # coarse samples of f(r, th) = 3 + 0.5 r (r = fine ring index) at the coarse centres
    centres = (np.arange(rings // rs) + 0.5) * rs - 0.5
    coarse = np.repeat(3.0 + 0.5 * centres, theta // ts)
    fine = np.asarray(U @ coarse).reshape(rings, theta)
    want = 3.0 + 0.5 * np.arange(rings, dtype=np.float64)
    inner = (np.arange(rings) >= centres[0]) & (np.arange(rings) <= centres[-1])
    np.testing.assert_allclose(fine[inner], np.broadcast_to(want[inner, None], fine[inner].shape), rtol=1e-6)
    # the reduce samples a function linear in the ring index at the centres
    R = np.kron(o.z_reduce.astype(np.float64), o.layer_reduce.astype(np.float64))
    f = np.repeat(want, theta)
    np.testing.assert_allclose(R @ f, coarse, rtol=1e-6)


def test_radial_builder_errors():
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso

    c = torch.from_numpy(_grid(10, 48))
    with pytest.raises(ValueError, match="not divisible by radial_stride"):
        cso.build_compton_sparse_projector_radial(c, 4, 4)
    with pytest.raises(ValueError, match="must be positive"):
        cso.build_compton_sparse_projector_radial(c, 0, 4)
    # rings of different lengths
    from jscc_recon_spect_cylinder_gb300 import synthetic

    a = synthetic.polar_grid(2, 48, 30.0).coor
    b = synthetic.polar_grid(4, 96, 60.0).coor
    mixed = torch.cat((a, b[b[:, 0] ** 2 + b[:, 1] ** 2 > 35.0 ** 2]), dim=0)
    with pytest.raises(ValueError, match="one length"):
        cso.build_compton_sparse_projector_radial(mixed, 1, 4)
    with pytest.raises(ValueError, match="one length"):
        osp.build_radial_projector(mixed.numpy(), 1, 4)
