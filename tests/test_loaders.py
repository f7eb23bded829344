"""On-disk formats (SysMat_polar, Sensi, CntStat, List and factor CSVs) against the
reference's own loading expressions (main_plane_sparse.py:296-329,
sparse_main_utils.py:123-127), on small files written here."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from jscc_recon_spect_cylinder_gb300 import loaders


def _sysmat_file(tmp_path, V=37, B=101, seed=0):
    a = np.random.default_rng(seed).random((V, B), dtype=np.float32)
    p = tmp_path / "SysMat_polar"
    a.tofile(p)
    return p, a


def test_sysmat_polar_cpu_matches_reference_expression(tmp_path):
    p, a = _sysmat_file(tmp_path)
    got = loaders.load_sysmat_polar(p, 37, device="cpu", intensity=2.5)
    ref = torch.from_numpy(np.fromfile(p, dtype=np.float32).reshape(37, -1).T.copy()) * 2.5
    assert got.shape == (101, 37) and torch.equal(got, ref)
    with pytest.raises(ValueError):
        loaders.load_sysmat_polar(p, 36, device="cpu")


def test_small_formats(tmp_path):
    rng = np.random.default_rng(1)
    s = rng.random(37, dtype=np.float32)
    s.tofile(tmp_path / "Sensi_s")
    got = loaders.load_sensitivity(tmp_path / "Sensi_s", 37, intensity=0.5)
    assert got.shape == (37, 1) and torch.equal(got, torch.from_numpy(s.reshape(37, 1)) * 0.5)
    cnt = rng.integers(0, 50, size=(3, 20)).astype(np.float32)
    np.savetxt(tmp_path / "cnt.csv", cnt, delimiter=",")
    proj = loaders.load_cntstat(tmp_path / "cnt.csv", 3)
    assert proj.shape == (20, 3) and torch.equal(proj, torch.from_numpy(cnt.T.copy()))
    lst = np.array([[5, 0.1, 700, 0.4, 9.9], [6, 0.2, 701, 0.3, 9.9]], dtype=np.float32)
    np.savetxt(tmp_path / "1.csv", lst, delimiter=",")
    np.savetxt(tmp_path / "2.csv", lst[:1], delimiter=",")
    assert torch.equal(loaders.load_list_csv(tmp_path / "1.csv"), torch.from_numpy(lst[:, :4]))
    one = loaders.load_list_csv(tmp_path / "2.csv")
    assert one.shape == (1, 4) and torch.equal(one, torch.from_numpy(lst[:1, :4]))
    det = np.concatenate((np.arange(4, dtype=np.float32)[:, None], rng.random((4, 3), dtype=np.float32)), axis=1)
    np.savetxt(tmp_path / "det.csv", det, delimiter=",")
    coor = rng.random((37, 3), dtype=np.float32)
    np.savetxt(tmp_path / "coor_polar_full.csv", coor, delimiter=",")
    rot = np.stack([np.roll(np.arange(1, 38), k) for k in range(2)], axis=1)
    np.savetxt(tmp_path / "RotMat_full.csv", rot, delimiter=",", fmt="%d")
    np.savetxt(tmp_path / "RotMatInv_full.csv", rot, delimiter=",", fmt="%d")
    d, c, r, ri = loaders.load_factors(tmp_path, tmp_path / "det.csv")
    assert torch.allclose(d, torch.from_numpy(det[:, 1:4])) and torch.allclose(c, torch.from_numpy(coor))
    assert r.dtype == torch.int64 and torch.equal(r, torch.from_numpy(rot))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_sysmat_polar_gpu_transpose(cuda, tmp_path, dtype):
    """GPU-side transpose/scale/cast in column blocks equals the reference's host expression."""
    p, a = _sysmat_file(tmp_path, V=300, B=1000, seed=3)
    got = loaders.load_sysmat_polar(p, 300, device=cuda, intensity=1.5, dtype=dtype, block_bins=256)
    ref = (torch.from_numpy(a.T.copy()) * 1.5).to(dtype)
    assert got.device.type == "cuda" and got.dtype == dtype and got.is_contiguous()
    assert torch.equal(got.cpu(), ref)
