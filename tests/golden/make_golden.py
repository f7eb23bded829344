"""Generate the golden fixtures by running the REFERENCE's own functions on CPU.

Run in a container where the reference checkout is readable (it is imported from
REF_DIR below, never copied). Inputs are seeded synthetic problems from
jscc_recon_spect_cylinder_gb300.synthetic; each fixture stores inputs and the
reference's outputs in one .npz so tests can replay them without the reference.

    python tests/golden/make_golden.py [--ref /root/reference] [--only NAME ...]
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from jscc_recon_spect_cylinder_gb300 import synthetic  # noqa: E402


def _np(t):
    return t.detach().cpu().numpy()


def save(name, **arrays):
    path = HERE / f"{name}.npz"
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print(f"wrote {path.name}: " + ", ".join(f"{k}{tuple(np.asarray(v).shape)}" for k, v in arrays.items()))


# ----------------------------------------------------------------------------- SC
def golden_sc(ref):
    """osem_bin_mode (R-form, 2 energies, 3 subsets, 2 iterations), get_weight_single,
    split_tensor_even and osem_bin_mode_local with a CPU-generator permutation."""
    rop = ref["recon_osem_plane"]
    loc = ref["recon_osem_local_cntstat"]
    torch.manual_seed(1234)
    probs = [synthetic.sc_problem(n_r=6, n_theta=24, disk_radius=20.0, n_phi=48, views=4, flat=False,
                                  total_counts=2e4, seed=synthetic.SEED + e) for e in range(2)]
    R = probs[0].rotmat.size(1)
    V = probs[0].grid.n_vox
    B = probs[0].sysmat.size(0)
    S = 3
    perm = torch.randperm(B)
    subsets = rop.split_tensor_even(perm, S, dim=0)
    A_l = [[p.sysmat[ids] for p in probs] for ids in subsets]
    y_l = [[p.proj[ids] for p in probs] for ids in subsets]
    rot = [p.rotmat for p in probs]
    inv = [p.rotmat_inv for p in probs]
    s = probs[0].s_map + probs[1].s_map
    img = torch.ones((V, 1))
    imgs = []
    with torch.no_grad():
        for _ in range(2):
            img = rop.osem_bin_mode(A_l, y_l, rot, inv, img, s, R)
            imgs.append(img.clone())
        w1 = rop.get_weight_single(probs[0].sysmat, probs[0].proj[:, :1], torch.ones((V, 1)))
        w1_local = loc.get_weight_single(probs[0].sysmat, probs[0].proj[:, :1], torch.ones((V, 1)))
    split_cases = [(10, 3), (7, 7), (5, 8), (0, 3), (1024, 10)]
    split_bounds = []
    for n, k in split_cases:
        parts = rop.split_tensor_even(torch.arange(n), k, dim=0)
        split_bounds.append([int(p.numel()) for p in parts] + [-1] * (10 - k))
    # local variant with a CPU generator (device-specific permutations are replayed by tests)
    gen = torch.Generator(device="cpu")
    gen.manual_seed(20260331)
    A_full = [probs[0].sysmat]
    y_full = [probs[0].proj]
    img_l = torch.ones((V, 1))
    perms = []
    with torch.no_grad():
        for _ in range(2):
            g_state = gen.get_state()
            sl, pl = loc.build_random_bin_subsets(A_full, y_full, S, gen)
            gen2 = torch.Generator(device="cpu")
            gen2.set_state(g_state)
            perms.append(torch.randperm(B, generator=gen2))
            img_l = loc.osem_bin_mode_local(sl, pl, [rot[0]], [inv[0]], img_l, probs[0].s_map)
    save("sc_osem",
         A0=_np(probs[0].sysmat), A1=_np(probs[1].sysmat), y0=_np(probs[0].proj), y1=_np(probs[1].proj),
         rot0=_np(rot[0]), rot1=_np(rot[1]), inv0=_np(inv[0]), inv1=_np(inv[1]), s=_np(s),
         s0=_np(probs[0].s_map), perm=_np(perm), n_subsets=S, img_iter1=_np(imgs[0]), img_iter2=_np(imgs[1]),
         w_single=_np(w1), w_single_local=_np(w1_local), split_cases=np.array(split_cases),
         split_sizes=np.array(split_bounds), local_perms=np.stack([_np(p) for p in perms]),
         local_img_iter2=_np(img_l))


def golden_dense_compton(ref):
    """osem_list_mode / osem_joint_mode over stored dense T blocks, get_weight_compton
    and safe_em_update edge cases."""
    rop = ref["recon_osem_plane"]
    rsp = ref["recon_osem_plane_sparse"]
    prob = synthetic.sc_problem(n_r=5, n_theta=20, disk_radius=20.0, n_phi=40, views=4, flat=False,
                                total_counts=2e4, seed=synthetic.SEED + 7)
    V = prob.grid.n_vox
    R = prob.rotmat.size(1)
    g = torch.Generator().manual_seed(99)
    S, D = 2, 2
    t_all = []
    for _ in range(R):
        t = torch.rand((37, V), generator=g) ** 4
        t_all.append(t / t.sum(dim=1, keepdim=True))
    t_list = [[[[None] for _ in range(D)] for _ in range(R)] for _ in range(S)]
    for i in range(R):
        for j, ts in enumerate(rop.split_tensor_even(t_all[i], S, dim=0)):
            for k, tk in enumerate(rop.split_tensor_even(ts, D, dim=0)):
                t_list[j][i][k][0] = tk
    B = prob.sysmat.size(0)
    subsets = rop.split_tensor_even(torch.arange(B), S, dim=0)
    A_l = [[prob.sysmat[ids]] for ids in subsets]
    y_l = [[prob.proj[ids]] for ids in subsets]
    s_d = torch.rand((V, 1), generator=g) + 0.5
    with torch.no_grad():
        img_list = rop.osem_list_mode(t_list, [prob.rotmat], [prob.rotmat_inv], torch.ones((V, 1)), s_d, R)
        img_joint = rop.osem_joint_mode(A_l, y_l, t_list, [prob.rotmat], [prob.rotmat_inv], torch.ones((V, 1)),
                                        0.5 * prob.s_map + 1.5 * s_d, 0.5, R)
        w_c = rop.get_weight_compton(t_all[0], torch.ones((V, 1)))
        w = torch.tensor([[1.0], [float("nan")], [float("inf")], [-2.0], [3.0], [4.0], [5.0]])
        sm = torch.tensor([[2.0], [1.0], [1.0], [1.0], [0.0], [float("nan")], [1e-13]])
        im = torch.full((7, 1), 3.0)
        safe = rsp.safe_em_update(im, w, sm)
    save("dense_compton",
         A=_np(prob.sysmat), y=_np(prob.proj), rot=_np(prob.rotmat), inv=_np(prob.rotmat_inv), s=_np(prob.s_map),
         s_d=_np(s_d), t=np.stack([_np(t) for t in t_all]), n_subsets=S, n_divide=D, img_list=_np(img_list),
         img_joint=_np(img_joint), w_compton=_np(w_c), safe_img=_np(im), safe_w=_np(w), safe_s=_np(sm),
         safe_out=_np(safe))


GENERATORS = {
    "sc_osem": golden_sc,
    "dense_compton": golden_dense_compton,
}


def load_reference(ref_dir: Path):
    sys.path.insert(0, str(ref_dir))
    import importlib

    mods = {}
    for name in ("recon_osem_plane", "recon_osem_plane_sparse", "recon_osem_local_cntstat",
                 "recon_osem_local_sparse_jsccsd_only", "compton_sparse_ops", "process_list_plane_strict",
                 "process_list_plane_sparse", "process_list_plane"):
        mods[name] = importlib.import_module(name)
    return mods


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    torch.set_num_threads(1)
    ref = load_reference(Path(args.ref))
    for name, fn in GENERATORS.items():
        if args.only and name not in args.only:
            continue
        fn(ref)


if __name__ == "__main__":
    main()
