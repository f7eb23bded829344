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


# ----------------------------------------------------------------------------- Compton
def _planar_detector_subset(ref_dir: Path, per_layer=48, seed=5):
    """A subset of the shipped 4-layer planar detector (Factors/511keV_RotateNum10/Detector.csv):
    `per_layer` pixels from each |y| layer, so the strict crystal-variance branch applies."""
    det = np.genfromtxt(ref_dir / "Factors" / "511keV_RotateNum10" / "Detector.csv", delimiter=",",
                        dtype=np.float32)[:, 1:4]
    rng = np.random.default_rng(seed)
    layers = np.unique(np.abs(det[:, 1]))
    pick = []
    for y in layers:
        ids = np.nonzero(np.abs(det[:, 1]) == y)[0]
        pick.append(rng.choice(ids, per_layer, replace=False))
    return det[np.sort(np.concatenate(pick))]


def _cylinder_detector(n_phi=24, n_axial=2):
    scat = synthetic.cylinder_pixels(120.0, n_phi, n_axial, 4.0).float().numpy()
    absb = synthetic.cylinder_pixels(150.0, n_phi, n_axial, 4.0).float().numpy()
    return np.concatenate((scat, absb), axis=0).astype(np.float32), scat.shape[0]


def _events(det, n_front, E, e0, seed):
    """Seeded list (cp1, e1, cp2, e2), 1-based ids: first hit among the first n_front
    detectors, second hit among the rest; e1 from a Compton-like spread."""
    rng = np.random.default_rng(seed)
    cp1 = rng.integers(1, n_front + 1, E)
    cp2 = rng.integers(n_front + 1, det.shape[0] + 1, E)
    e1 = rng.uniform(0.06, 0.9 * (2 * e0 ** 2 / (0.511 + 2 * e0)), E)
    e2 = e0 - e1
    return np.stack((cp1, e1, cp2, e2), axis=1).astype(np.float32)


def golden_compton(ref):
    """Strict and legacy T builders on (a) a 4-layer planar detector subset of the shipped
    geometry and (b) a cylinder detector (isotropic-fallback sigma_pos)."""
    strict = ref["process_list_plane_strict"]
    legacy = ref["process_list_plane"]
    out = {}
    grid = synthetic.polar_grid(8, 24, 20.0)
    coor = grid.coor.numpy()
    for tag, (det, n_front), e0, dr in (
        ("planar", (_planar_detector_subset(REF_DIR), 96), 0.511, 0.0),
        ("cyl", _cylinder_detector(), 0.662, 0.5),
    ):
        g = torch.Generator().manual_seed(11)
        sysmat = (torch.rand((det.shape[0], coor.shape[0]), generator=g) * 1e-3).numpy()
        lst = _events(det, n_front, 160, e0, seed=len(tag))
        res = 0.1 * (0.662 / e0) ** 0.5
        tmax = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
        args = (dr, dr, e0, res, tmax, 0.05, e0 - 0.06)
        torch.manual_seed(77)
        L = torch.from_numpy(lst.copy())
        with torch.no_grad():
            t, tc, ts = strict.get_compton_backproj_list_single(torch.from_numpy(sysmat), torch.from_numpy(det),
                                                                torch.from_numpy(coor), L, *args, "cpu")
        smeared = L.numpy().copy()  # the strict builder smears the caller's list in place
        torch.manual_seed(77)
        n1 = torch.randn(lst.shape[0]).numpy()
        n2 = torch.randn(lst.shape[0]).numpy()
        torch.manual_seed(78)
        L2 = torch.from_numpy(lst.copy())
        with torch.no_grad():
            lt, ltc, lts = legacy.get_compton_backproj_list_single(torch.from_numpy(sysmat), torch.from_numpy(det),
                                                                   torch.from_numpy(coor), L2, 1.0 + dr, 1.0 + dr,
                                                                   e0, res, tmax, 0.05, e0 - 0.06, "cpu")
        out.update({f"{tag}_det": det, f"{tag}_sysmat": sysmat, f"{tag}_list": lst, f"{tag}_smeared": smeared,
                    f"{tag}_noise1": n1, f"{tag}_noise2": n2, f"{tag}_args": np.array(args),
                    f"{tag}_t": t.numpy(), f"{tag}_tc": tc.numpy(), f"{tag}_ts": ts.numpy(),
                    f"{tag}_legacy_smeared": L2.numpy().copy(), f"{tag}_legacy_t": lt.numpy(),
                    f"{tag}_legacy_tc": ltc.numpy(), f"{tag}_legacy_ts": lts.numpy()})
    save("compton_builders", coor=coor, **out)


def golden_sparse(ref):
    """Sparse projector on the shipped 511keV_RotateNum10 grid and on a small synthetic grid
    (stride reduction), its operators, the sparse builder and both sparse weights."""
    cso = ref["compton_sparse_ops"]
    rsp = ref["recon_osem_plane_sparse"]
    loc = ref["recon_osem_local_sparse_jsccsd_only"]
    psp = ref["process_list_plane_sparse"]
    out = {}
    coor_r10 = torch.from_numpy(np.genfromtxt(REF_DIR / "Factors" / "511keV_RotateNum10" / "coor_polar_full.csv",
                                              delimiter=",", dtype=np.float32))
    p10 = cso.build_compton_sparse_projector(coor_r10, theta_stride=2, z_stride=2, rotate_num=10)
    g = torch.Generator().manual_seed(3)
    rows = torch.rand((3, p10.coarse_pixel_num), generator=g)
    frows = torch.rand((3, p10.fine_pixel_num), generator=g)
    img_f = torch.rand((p10.fine_pixel_num, 1), generator=g)
    img_c = torch.rand((p10.coarse_pixel_num, 1), generator=g)
    for name in ("layer_reduce", "layer_expand", "z_reduce", "z_expand"):
        m = getattr(p10, name).numpy()
        nz = np.nonzero(m)
        out[f"r10_{name}_idx"] = np.stack(nz).astype(np.int32)
        out[f"r10_{name}_val"] = m[nz]
        out[f"r10_{name}_shape"] = np.array(m.shape)
    rotmat = np.genfromtxt(REF_DIR / "Factors" / "511keV_RotateNum10" / "RotMat_full.csv", delimiter=",",
                           dtype=np.int64)
    rotinv = np.genfromtxt(REF_DIR / "Factors" / "511keV_RotateNum10" / "RotMatInv_full.csv", delimiter=",",
                           dtype=np.int64)
    out.update({
        "r10_rotmat": rotmat.astype(np.int32), "r10_rotmat_inv": rotinv.astype(np.int32),
        "r10_coor_full": coor_r10.numpy(), "r10_coor_coarse": p10.coor_coarse.numpy(),
        "r10_ring_strides": np.array(p10.ring_strides),
        "r10_dims": np.array([p10.fine_layer_num, p10.fine_z_num, p10.coarse_layer_num, p10.coarse_z_num]),
        "r10_rows_c": rows.numpy(), "r10_rows_f": frows.numpy(), "r10_img_f": img_f.numpy(),
        "r10_img_c": img_c.numpy(),
        "r10_up": cso.upsample_coarse_rows_to_fine(rows, p10).numpy(),
        "r10_adj": cso.project_fine_rows_to_coarse_adjoint(frows, p10).numpy(),
        "r10_red": cso.reduce_fine_rows_to_coarse(frows, p10).numpy(),
        "r10_img_red": cso.reduce_fine_image_to_coarse(img_f, p10).numpy(),
        "r10_img_up": cso.upsample_coarse_weight_to_fine(img_c, p10).numpy(),
    })
    # small synthetic grid: 6 rings x 24 theta x 4 z planes; theta stride 4 with 4 views -> 3
    planes = [synthetic.polar_grid(6, 24, 20.0, z=z).coor for z in (-6.0, -2.0, 2.0, 6.0)]
    coor = torch.cat(planes, dim=0)
    p = cso.build_compton_sparse_projector(coor, theta_stride=4, z_stride=2, rotate_num=4)
    det, n_front = _planar_detector_subset(REF_DIR, per_layer=32, seed=9), 64
    e0 = 0.511
    sysmat = (torch.rand((det.shape[0], coor.shape[0]), generator=g) * 1e-3)
    lst = _events(det, n_front, 200, e0, seed=21)
    res = 0.1 * (0.662 / e0) ** 0.5
    tmax = 2 * e0 ** 2 / (0.511 + 2 * e0) - 0.001
    args = (0.0, 0.0, e0, res, tmax, 0.05, e0 - 0.06)
    torch.manual_seed(91)
    with torch.no_grad():
        ev_rows, _, _ = psp.get_compton_backproj_list_single_sparse(sysmat, torch.from_numpy(det), p,
                                                                     torch.from_numpy(lst.copy()), *args, "cpu")
    torch.manual_seed(91)
    n1 = torch.randn(lst.shape[0])
    n2 = torch.randn(lst.shape[0])
    # the smeared list exactly as the sparse builder forms it on CPU (same torch expression,
    # process_list_plane_sparse.py:45-48), so tests can feed it to the inner builder
    Lt = torch.from_numpy(lst.copy())
    e1s = Lt[:, 1] + (Lt[:, 1] * res / 2.355 * (e0 / Lt[:, 1]) ** 0.5) * n1
    e2s = Lt[:, 3] + (Lt[:, 3] * res / 2.355 * (e0 / Lt[:, 3]) ** 0.5) * n2
    smeared = lst.copy()
    smeared[:, 1] = e1s.numpy()
    smeared[:, 3] = e2s.numpy()
    n1, n2 = n1.numpy(), n2.numpy()
    x = torch.rand((coor.shape[0], 1), generator=g) + 0.2
    with torch.no_grad():
        t_fine, valid = cso.materialize_sparse_event_rows_to_fine(ev_rows, sysmat, p)
        w_grouped = rsp.get_weight_compton_sparse(ev_rows, sysmat, x, p)
        w_mat = loc.get_weight_compton_sparse(ev_rows, sysmat, x, p)
    out.update({
        "s_coor": coor.numpy(), "s_coor_coarse": p.coor_coarse.numpy(), "s_ring_strides": np.array(p.ring_strides),
        "s_dims": np.array([p.fine_layer_num, p.fine_z_num, p.coarse_layer_num, p.coarse_z_num]),
        "s_layer_expand": p.layer_expand.numpy(), "s_z_expand": p.z_expand.numpy(),
        "s_layer_reduce": p.layer_reduce.numpy(), "s_z_reduce": p.z_reduce.numpy(),
        "s_det": det, "s_sysmat": sysmat.numpy(), "s_list": lst, "s_smeared": smeared, "s_noise1": n1,
        "s_noise2": n2,
        "s_args": np.array(args), "s_event_rows": ev_rows.numpy(), "s_x": x.numpy(),
        "s_t_fine": t_fine.numpy(), "s_valid": valid.numpy(), "s_w_grouped": w_grouped.numpy(),
        "s_w_mat": w_mat.numpy(),
    })
    save("sparse_ops", **out)


def golden_sensitivity(ref):
    """Sensitivity builders: the Compton d of build_sparse_sensi_d_local
    (main_local_sparse_jsccsd_only.py:95-108; build_sparse_sensi_d, main_plane_sparse.py:214-231,
    is the same sum followed by a rescale, and pins "cuda:0") on the sparse_ops fixture's rows
    split into two rotation blocks, and the SC sensitivity of compute_sensitivity_local
    (main_local_cntstat.py:140-146, the same formula as main_plane_sparse.py:440-444) on the
    shipped 10-view rotation tables."""
    import importlib

    cso = ref["compton_sparse_ops"]
    msp = importlib.import_module("main_local_sparse_jsccsd_only")
    mcs = importlib.import_module("main_local_cntstat")
    sp = np.load(Path(__file__).parent / "sparse_ops.npz")
    coor = torch.from_numpy(sp["s_coor"])
    p = cso.build_compton_sparse_projector(coor, theta_stride=4, z_stride=2, rotate_num=4)
    rows = torch.from_numpy(sp["s_event_rows"])
    sysmat = torch.from_numpy(sp["s_sysmat"])
    half = rows.size(0) // 2
    with torch.no_grad():
        d = msp.build_sparse_sensi_d_local([[rows[:half], rows[half:]]], [sysmat], [p], coor.size(0),
                                           torch.device("cpu"), block_size=16)
    rotinv = torch.from_numpy(np.genfromtxt(REF_DIR / "Factors" / "511keV_RotateNum10" / "RotMatInv_full.csv",
                                            delimiter=",", dtype=np.int64))
    g = torch.Generator().manual_seed(17)
    # an SC matrix of exact float32 values k * 2^-18 (k < 256) stored as its uint8 codes
    codes = torch.randint(0, 256, (32, rotinv.size(0)), generator=g, dtype=torch.uint8)
    sc_sysmat = codes.to(torch.float32) * 2.0 ** -18
    with torch.no_grad():
        s = mcs.compute_sensitivity_local(sc_sysmat, rotinv, 10)
    save("sensitivity", d_rows=rows.numpy(), d_half=np.array(half), d_local=d.numpy(),
         sc_codes=codes.numpy(), sc_s=s.numpy())  # rotation tables: sparse_ops r10_rotmat_inv


# ----------------------------------------------------------------------------- runners
class _CudaAsCpu:
    """Runs the reference's runners, which pin "cuda:0" (recon_osem_plane.py:168-171,
    recon_osem_plane_sparse.py:150-153), on the CPU: every tensor / projector move to a CUDA
    device stays on the CPU, the T-memory budget is unbounded (so nothing is pinned) and the
    GPU memory report is skipped. The runners' own code (staging, permutation, phase order,
    snapshots, save_img) runs unchanged."""

    def __init__(self, ref):
        self.mods = [ref["recon_osem_plane"], ref["recon_osem_plane_sparse"]]

    @staticmethod
    def _cuda(a):
        return (isinstance(a, str) and a.startswith("cuda")) or (isinstance(a, torch.device) and a.type == "cuda")

    def __enter__(self):
        self.orig_to = torch.Tensor.to
        orig_to = self.orig_to
        cuda = self._cuda

        def to(t, *args, **kwargs):
            args = tuple("cpu" if cuda(a) else a for a in args)
            if cuda(kwargs.get("device")):
                kwargs["device"] = "cpu"
            return orig_to(t, *args, **kwargs)

        torch.Tensor.to = to
        self.saved = []
        for m in self.mods:
            for name, fn in (("get_t_budget_bytes_per_gpu", lambda n: [1 << 62] * n),
                             ("get_gpu_memory_usage", lambda n: None)):
                self.saved.append((m, name, getattr(m, name)))
                setattr(m, name, fn)
        return self

    def __exit__(self, *exc):
        torch.Tensor.to = self.orig_to
        for m, name, fn in self.saved:
            setattr(m, name, fn)
        return False


def _read_images(path, names):
    return {n: np.fromfile(path / n, dtype=np.float32) for n in names}


def golden_runners(ref):
    """The reference's four runners on small seeded problems, with the files they write:
    run_recon_osem (dense T, recon_osem_plane.py:161-403) and run_recon_osem_sparse
    (recon_osem_plane_sparse.py:144-348) on one GPU's path, run on the CPU through
    _CudaAsCpu; run_recon_osem_local_cntstat (recon_osem_local_cntstat.py:56-100) and
    run_recon_osem_local_sparse_jsccsd_only (recon_osem_local_sparse_jsccsd_only.py:111-202)
    with device=cpu. Two energies, two rotations, 3 subsets, 2 divides, snapshots every 2
    iterations. The global and per-runner permutations are recorded so that tests replay
    them (the local runners draw theirs on the device they run on)."""
    import tempfile
    from types import SimpleNamespace

    rop = ref["recon_osem_plane"]
    rsp = ref["recon_osem_plane_sparse"]
    cso = ref["compton_sparse_ops"]
    lcs = ref["recon_osem_local_cntstat"]
    ljs = ref["recon_osem_local_sparse_jsccsd_only"]
    E, R, S, D = 2, 2, 3, 2
    probs = [synthetic.sc_problem(n_r=6, n_theta=24, disk_radius=20.0, n_phi=48, views=R, flat=False,
                                  total_counts=2e4, seed=synthetic.SEED + 10 + e) for e in range(E)]
    V = probs[0].grid.n_vox
    B = probs[0].sysmat.size(0)
    g = torch.Generator().manual_seed(404)
    sysmat = [p.sysmat.clone() for p in probs]
    rot = [p.rotmat.clone() for p in probs]
    inv = [p.rotmat_inv.clone() for p in probs]
    proj = [p.proj.clone() for p in probs]
    proj_d = [torch.poisson(p.proj, generator=g) for p in probs]
    s = sum(p.s_map for p in probs)
    d = torch.rand((V, 1), generator=g) + 0.5
    # dense T per energy and rotation (normalised rows, uneven counts)
    t_dense = []
    for e in range(E):
        blocks = []
        for r in range(R):
            t = torch.rand((23 + 7 * e + 3 * r, V), generator=g) ** 4
            blocks.append(t / t.sum(dim=1, keepdim=True))
        t_dense.append(blocks)
    # sparse packed rows per energy and rotation (cp1 indexes the SC matrix rows, 1-based)
    proj_sp = cso.build_compton_sparse_projector(probs[0].grid.coor, theta_stride=4, z_stride=1, rotate_num=R)
    vc = proj_sp.coarse_pixel_num
    t_sparse = []
    for e in range(E):
        blocks = []
        for r in range(R):
            n = 31 + 5 * e + 4 * r
            cp1 = torch.randint(1, B + 1, (n,), generator=g)
            tc = torch.rand((n, vc), generator=g) ** 3
            blocks.append(cso.pack_sparse_event_rows(cp1, tc))
        t_sparse.append(blocks)
    iter_arg = SimpleNamespace(sc=4, jsccd=4, jsccsd=4, save_iter_step=2, osem_subset_num=S, t_divide_num=D,
                               ene_num=E, mode=0, seed=20260331)
    alpha = 0.5
    names = ["Image_SC", "Image_SCD", "Image_JSCCD", "Image_JSCCSD", "Image_SC_Iter_4_2", "Image_SCD_Iter_4_2",
             "Image_JSCCD_Iter_4_2", "Image_JSCCSD_Iter_4_2"]
    out = {}
    with tempfile.TemporaryDirectory() as tmp, torch.no_grad():
        tmp = Path(tmp)
        for tag, runner, t_all, extra in (("dense", rop.run_recon_osem, t_dense, ()),
                                          ("sparse", rsp.run_recon_osem_sparse, t_sparse, ([proj_sp, proj_sp],))):
            torch.manual_seed(2718)
            perm = torch.randperm(B)
            torch.manual_seed(2718)
            smap = SimpleNamespace(s=s.clone(), d=d.clone())
            path = tmp / tag
            path.mkdir()
            with _CudaAsCpu(ref):
                runner([a.clone() for a in sysmat], [r.clone() for r in rot], [r.clone() for r in inv],
                       [p.clone() for p in proj], [p.clone() for p in proj_d], [[t.clone() for t in ts] for ts in t_all],
                       *extra, iter_arg, smap, alpha, str(path) + "/", 1)
            for n, a in _read_images(path, names).items():
                out[f"{tag}_{n}"] = a
            out[f"{tag}_perm"] = perm.numpy()
        # local runners: device = cpu, CPU generator; the permutations of every iteration
        for tag in ("cntstat", "jsccsd"):
            gen = torch.Generator().manual_seed(iter_arg.seed)
            n_it = iter_arg.sc if tag == "cntstat" else iter_arg.jsccsd
            out[f"{tag}_perms"] = np.stack([torch.randperm(B, generator=gen).numpy() for _ in range(n_it)])
        path = tmp / "cntstat"
        path.mkdir()
        try:
            lcs.run_recon_osem_local_cntstat([a.clone() for a in sysmat], [r.clone() for r in rot],
                                             [r.clone() for r in inv], [p.clone() for p in proj], iter_arg,
                                             SimpleNamespace(s=s.clone()), str(path) + "/", torch.device("cpu"))
        except NameError:
            pass  # the runner returns an undefined name after writing its files (recon_osem_local_cntstat.py:100)
        for n, a in _read_images(path, ["Image_SC", "Image_SC_Iter_4_2"]).items():
            out[f"cntstat_{n}"] = a
        path = tmp / "jsccsd"
        path.mkdir()
        j = alpha * s + (2 - alpha) * d
        t_local = [[t.clone() for t in ts] for ts in t_sparse]
        ljs.run_recon_osem_local_sparse_jsccsd_only([a.clone() for a in sysmat], [a.clone() for a in sysmat],
                                                    [r.clone() for r in rot], [r.clone() for r in inv],
                                                    [p.clone() for p in proj], t_local, [proj_sp, proj_sp], iter_arg,
                                                    SimpleNamespace(j=j.clone()), alpha, str(path) + "/",
                                                    torch.device("cpu"))
        for n, a in _read_images(path, ["Image_JSCCSD", "Image_JSCCSD_Iter_4_2"]).items():
            out[f"jsccsd_{n}"] = a
    save("runners", sysmat=np.stack([_np(a) for a in sysmat]), rot=np.stack([_np(r) for r in rot]),
         inv=np.stack([_np(r) for r in inv]), proj=np.stack([_np(p) for p in proj]),
         proj_d=np.stack([_np(p) for p in proj_d]), s=_np(s), d=_np(d), coor=_np(probs[0].grid.coor),
         **{f"t_dense_{e}_{r}": _np(t_dense[e][r]) for e in range(E) for r in range(R)},
         **{f"t_sparse_{e}_{r}": _np(t_sparse[e][r]) for e in range(E) for r in range(R)},
         iter_arg=np.array([iter_arg.sc, iter_arg.jsccd, iter_arg.jsccsd, iter_arg.save_iter_step, S, D, E]),
         alpha=np.array(alpha), **out)


GENERATORS = {
    "sc_osem": golden_sc,
    "dense_compton": golden_dense_compton,
    "compton_builders": golden_compton,
    "sparse_ops": golden_sparse,
    "sensitivity": golden_sensitivity,
    "runners": golden_runners,
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


REF_DIR = Path("/root/reference")


def main():
    global REF_DIR
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=str(REF_DIR))
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    REF_DIR = Path(args.ref)
    torch.set_num_threads(1)
    ref = load_reference(Path(args.ref))
    for name, fn in GENERATORS.items():
        if args.only and name not in args.only:
            continue
        fn(ref)


if __name__ == "__main__":
    main()
