"""Host side of the batched path (CPU): the bin-permuted subset layout and the BF16 hi / lo
representation of the instance vectors."""
from __future__ import annotations

import torch


def test_subset_blocks_cover_every_bin_once():
    from jscc_recon_spect_cylinder_gb300 import batched
    from jscc_recon_spect_cylinder_gb300.recon_osem_plane import split_tensor_even

    B = 1001
    subsets = split_tensor_even(torch.randperm(B, generator=torch.Generator().manual_seed(2)), 7)
    blocks, perm = batched.subset_blocks(subsets)
    assert len(blocks) == 7
    off = 0
    for (b0, nb, nbp), ids in zip(blocks, subsets):
        assert b0 == off and nb == ids.numel() and nbp % 8 == 0 and nbp - nb < 8
        assert torch.equal(perm[b0:b0 + nb], ids)
        assert torch.all(perm[b0 + nb:b0 + nbp] == -1)
        off += nbp
    real = perm[perm >= 0]
    assert torch.equal(torch.sort(real).values, torch.arange(B))
    # the inverse map the joint batch uses to remap efficiency-row ids
    inv = torch.full((B,), -1, dtype=torch.int64)
    inv[perm[perm >= 0]] = torch.arange(perm.numel())[perm >= 0]
    assert torch.equal(perm[inv], torch.arange(B))


def test_hi_lo_bf16_pairs_keep_sixteen_bits():
    """v = bf16(v) + bf16(v - bf16(v)) to ~2^-16 relative (the batch kernels' split): the
    instance vectors lose only ~1.5e-5 relative, far below the BF16 matrix's rounding."""
    g = torch.Generator().manual_seed(3)
    v = torch.exp(torch.randn(100000, generator=g) * 5)  # values spanning many orders of magnitude
    hi = v.to(torch.bfloat16)
    lo = (v - hi.float()).to(torch.bfloat16)
    rel = ((hi.float() + lo.float()) - v).abs() / v
    assert float(rel.max()) < 2.0 ** -16
    assert float((hi.float() - v).abs().div(v).max()) > 2.0 ** -10  # BF16 alone would not do
