"""GPU parity of the sensitivity builders (SC column sums through the inverse rotations and
the Compton d) against the reference's own outputs (tests/golden/sensitivity.npz) and the
oracle. Tolerance: relative L2 <= 1e-5 (float32 sums in a different order)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import osem_sc
from oracle import sparse as osp

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _sc_inputs(golden, cuda):
    g = golden("sensitivity")
    sp = golden("sparse_ops")
    A = torch.from_numpy(g["sc_codes"].astype(np.float32) * np.float32(2.0 ** -18)).to(cuda)
    rotinv = torch.from_numpy(sp["r10_rotmat_inv"].astype(np.int64)).to(cuda)
    return g, A, rotinv


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_sc_sensitivity_matches_reference(cuda, golden, dtype):
    """compute_sensitivity_local over the shipped 10-view inverse rotations; the matrix's
    values k * 2^-18 are exact in BF16, so both storages give the reference's sums."""
    from jscc_recon_spect_cylinder_gb300 import sensitivity

    g, A, rotinv = _sc_inputs(golden, cuda)
    s = sensitivity.compute_sensitivity_local(A.to(dtype), rotinv, 10)
    assert s.device.type == "cpu" and s.shape == (A.size(1), 1)
    assert rel_l2(s, g["sc_s"]) < TOL


def test_sc_sensitivity_row_subset_and_identity(cuda, golden):
    from jscc_recon_spect_cylinder_gb300 import ops

    g, A, rotinv = _sc_inputs(golden, cuda)
    ids = torch.tensor([3, 0, 17, 31, 8], device=cuda)
    s = ops.sc_sensitivity(A, rotinv, 4, row_idx=ids)
    ref = osem_sc.sc_sensitivity(A[ids].cpu().numpy(), rotinv.cpu().numpy(), 4)
    assert rel_l2(s.cpu(), ref) < TOL
    s1 = ops.sc_sensitivity(A)  # identity rotation: plain column sums
    assert rel_l2(s1.cpu(), A.cpu().double().sum(0, keepdim=True).t()) < TOL


def test_sparse_sensitivity_matches_reference(cuda, golden):
    """build_sparse_sensi_d_local on two rotation blocks of the fixture's sparse rows (a
    two-plane grid with z taps), and build_sparse_sensi_d's rescale."""
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import sensitivity

    g = golden("sensitivity")
    sp = golden("sparse_ops")
    p = cso.build_compton_sparse_projector(torch.from_numpy(sp["s_coor"]), 4, 2, 4)
    rows = torch.from_numpy(g["d_rows"])
    half = int(g["d_half"])
    sysmat = torch.from_numpy(sp["s_sysmat"])
    V = sysmat.size(1)
    d = sensitivity.build_sparse_sensi_d_local([[rows[:half], rows[half:]]], [sysmat], [p], V, cuda)
    assert d.device.type == "cpu"
    assert rel_l2(d, g["d_local"]) < TOL
    s_map_s = torch.rand((V, 1), generator=torch.Generator().manual_seed(2))
    r = sensitivity.build_sparse_sensi_d([[rows[:half], rows[half:]]], [sysmat], [p], s_map_s, 1000, 250)
    ref = osp.sensitivity_d_rescale(g["d_local"], s_map_s.numpy(), 1000, 250)
    assert rel_l2(r, ref) < TOL
    # no valid event: d stays zero and is not rescaled
    empty = torch.zeros((0, rows.size(1)))
    z = sensitivity.build_sparse_sensi_d([[empty]], [sysmat], [p], s_map_s, 10, 10)
    assert torch.count_nonzero(z) == 0


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_sc_sensitivity_sums_are_compensated(cuda, dtype):
    """Column sums of 300,000 rows whose values span 1e-8 .. 1 (a large leading term, then
    many small ones): the Kahan-compensated sums stay within 2.5e-7 relative of the exact
    float64 sums of the stored values (one float32 accumulator per column drifts by ~1e-5 here)."""
    from jscc_recon_spect_cylinder_gb300 import ops

    g = torch.Generator().manual_seed(12)
    B, V = 300_000, 24
    A = torch.rand((B, V), generator=g) ** 6
    A[0] = 1.0
    A = A.to(dtype)
    exact = A.double().sum(0)
    s = ops.sc_sensitivity(A.to(cuda)).cpu().double().ravel()
    assert float(((s - exact).abs() / exact).max()) < 2.5e-7
