"""The runner layer, the functions the reference's entry points call: every image file the
mirrored runners write (names, sizes, values) against the files the reference's own runners
wrote for the same inputs (tests/golden/runners.npz, made by tests/golden/make_golden.py):

* run_recon_osem (recon_osem_plane.py:161-403): SC, SC-D, dense-T JSCC-D and JSCC-SD phases
* run_recon_osem_sparse (recon_osem_plane_sparse.py:144-348): the same with packed sparse rows
* run_recon_osem_local_cntstat (recon_osem_local_cntstat.py:56-100)
* run_recon_osem_local_sparse_jsccsd_only (recon_osem_local_sparse_jsccsd_only.py:111-202)

Two energies, two rotations, 3 subsets, 2 divides, 4 iterations per phase, snapshots every 2.
The bin permutations the reference drew are replayed: the global one of the GPU runners
(torch.randperm on the CPU generator) and the per-iteration ones of the local runners (drawn
on the device they run on, so a CUDA run draws different ones than the CPU run that made the
fixture). Float32 path: relative L2 <= 1e-5 per image and per snapshot."""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
NAMES = ["Image_SC", "Image_SCD", "Image_JSCCD", "Image_JSCCSD", "Image_SC_Iter_4_2", "Image_SCD_Iter_4_2",
         "Image_JSCCD_Iter_4_2", "Image_JSCCSD_Iter_4_2"]


def _inputs(g):
    E = int(g["iter_arg"][6])
    R = g["rot"].shape[2]
    t = lambda kind: [[torch.from_numpy(g[f"t_{kind}_{e}_{r}"]) for r in range(R)] for e in range(E)]
    it = g["iter_arg"]
    iter_arg = SimpleNamespace(sc=int(it[0]), jsccd=int(it[1]), jsccsd=int(it[2]), save_iter_step=int(it[3]),
                               osem_subset_num=int(it[4]), t_divide_num=int(it[5]), ene_num=E, mode=0,
                               seed=20260331)
    return dict(sysmat=[torch.from_numpy(a) for a in g["sysmat"]], rot=[torch.from_numpy(r) for r in g["rot"]],
                inv=[torch.from_numpy(r) for r in g["inv"]], proj=[torch.from_numpy(p) for p in g["proj"]],
                proj_d=[torch.from_numpy(p) for p in g["proj_d"]], s=torch.from_numpy(g["s"]),
                d=torch.from_numpy(g["d"]), t_dense=t("dense"), t_sparse=t("sparse"), iter_arg=iter_arg,
                alpha=float(g["alpha"]), coor=torch.from_numpy(g["coor"]))


def _check_files(path: Path, g, tag, names):
    written = sorted(p.name for p in path.iterdir())
    assert written == sorted(names), written
    V = g["s"].shape[0]
    for n in names:
        got = np.fromfile(path / n, dtype=np.float32)
        ref = g[f"{tag}_{n}"]
        assert got.shape == ref.shape, (n, got.shape, ref.shape)
        for k in range(got.size // V):  # each snapshot row on its own
            err = rel_l2(got[k * V:(k + 1) * V], ref[k * V:(k + 1) * V])
            assert err < TOL, (n, k, err)


def _replay_randperm(monkeypatch, perm):
    orig = torch.randperm

    def randperm(n, *args, **kwargs):
        if n == perm.size and not args and not kwargs:
            return torch.from_numpy(perm.copy())
        return orig(n, *args, **kwargs)

    monkeypatch.setattr(torch, "randperm", randperm)


@pytest.mark.parametrize("tag", ["dense", "sparse"])
def test_gpu_runners_write_the_reference_files(cuda, golden, tmp_path, monkeypatch, tag):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane as rop
    from jscc_recon_spect_cylinder_gb300 import recon_osem_plane_sparse as rsp

    g = golden("runners")
    x = _inputs(g)
    _replay_randperm(monkeypatch, g[f"{tag}_perm"])
    smap = SimpleNamespace(s=x["s"].clone(), d=x["d"].clone())
    if tag == "dense":
        rop.run_recon_osem(x["sysmat"], x["rot"], x["inv"], x["proj"], x["proj_d"], x["t_dense"], x["iter_arg"],
                           smap, x["alpha"], str(tmp_path) + "/", 1)
    else:
        p = cso.build_compton_sparse_projector(x["coor"], theta_stride=4, z_stride=1, rotate_num=x["rot"][0].size(1))
        rsp.run_recon_osem_sparse(x["sysmat"], x["rot"], x["inv"], x["proj"], x["proj_d"], x["t_sparse"], [p, p],
                                  x["iter_arg"], smap, x["alpha"], str(tmp_path) + "/", 1)
    _check_files(tmp_path, g, tag, NAMES)


def _replay_local_perms(monkeypatch, perms):
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_cntstat as lcs
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_sparse_jsccsd_only as ljs

    calls = iter(range(perms.shape[0]))

    def subsets(n, subset_num, generator, device):
        perm = torch.from_numpy(perms[next(calls)].copy()).to(device)
        assert perm.numel() == n
        return list(torch.chunk(perm, subset_num, dim=0))

    monkeypatch.setattr(lcs, "random_bin_subset_ids", subsets)
    monkeypatch.setattr(ljs, "random_bin_subset_ids", subsets)


def test_local_cntstat_runner_writes_the_reference_files(cuda, golden, tmp_path, monkeypatch):
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_cntstat as lcs

    g = golden("runners")
    x = _inputs(g)
    _replay_local_perms(monkeypatch, g["cntstat_perms"])
    lcs.run_recon_osem_local_cntstat(x["sysmat"], x["rot"], x["inv"], x["proj"], x["iter_arg"],
                                     SimpleNamespace(s=x["s"].clone()), str(tmp_path) + "/", cuda)
    _check_files(tmp_path, g, "cntstat", ["Image_SC", "Image_SC_Iter_4_2"])


def test_local_jsccsd_runner_writes_the_reference_files(cuda, golden, tmp_path, monkeypatch):
    from jscc_recon_spect_cylinder_gb300 import compton_sparse_ops as cso
    from jscc_recon_spect_cylinder_gb300 import recon_osem_local_sparse_jsccsd_only as ljs

    g = golden("runners")
    x = _inputs(g)
    _replay_local_perms(monkeypatch, g["jsccsd_perms"])
    p = cso.build_compton_sparse_projector(x["coor"], theta_stride=4, z_stride=1, rotate_num=x["rot"][0].size(1))
    j = x["alpha"] * x["s"] + (2 - x["alpha"]) * x["d"]
    ljs.run_recon_osem_local_sparse_jsccsd_only(x["sysmat"], x["sysmat"], x["rot"], x["inv"], x["proj"],
                                                x["t_sparse"], [p, p], x["iter_arg"], SimpleNamespace(j=j),
                                                x["alpha"], str(tmp_path) + "/", cuda)
    _check_files(tmp_path, g, "jsccsd", ["Image_JSCCSD", "Image_JSCCSD_Iter_4_2"])
