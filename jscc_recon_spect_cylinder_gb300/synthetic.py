"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference ships no system matrices, projections or list files for its OSEM
path (Factors/*/SysMat_polar, CntStat/ and List/ are absent), so every input here is
synthetic. Generators are written with torch so they run on the CPU for small
parity cases and on the GPU for the full-size bench inputs; one seed gives one
workload on a given device type.

Geometry
 * Image: 2-D polar grid, ring-major (ring k at radius (k + 1/2) * dr, `n_theta`
   equally spaced angles starting at 0), one z plane — the consecutive-ring layout
   compton_sparse_ops._infer_polar_layout expects (compton_sparse_ops.py:59-92).
 * SC detector: pixels on a cylinder facing the axis. a_ij = cos(incidence) *
   pixel_area / (4 pi d^2) * exp(-mu * path_in_object) * lognormal(0, sigma).
 * Views: the detector turns by 2 pi v / R. The "flat" form stores all views as
   rows of one matrix (rotate_num = 1, identity rotation tables); the "rotated" form
   keeps one view's matrix and cyclic per-ring rotation tables (RotMat layout,
   1-based int64 [V, R]).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

SEED = 20260331  # reference default (main_plane_sparse.py:65)


@dataclass
class PolarGrid:
    n_r: int
    n_theta: int
    radius: float
    coor: torch.Tensor  # [V, 3] float32

    @property
    def n_vox(self) -> int:
        return self.n_r * self.n_theta


def polar_grid(n_r: int, n_theta: int, radius: float, z: float = 0.0, device="cpu") -> PolarGrid:
    dr = radius / n_r
    k = torch.arange(n_r, dtype=torch.float64, device=device)
    m = torch.arange(n_theta, dtype=torch.float64, device=device)
    rr = ((k + 0.5) * dr).unsqueeze(1).expand(n_r, n_theta)
    th = (2.0 * math.pi * m / n_theta).unsqueeze(0).expand(n_r, n_theta)
    coor = torch.stack((rr * torch.cos(th), rr * torch.sin(th), torch.full_like(rr, z)), dim=-1)
    return PolarGrid(n_r, n_theta, radius, coor.reshape(-1, 3).to(torch.float32))


def cyclic_rotation_tables(n_r: int, n_theta: int, rotate_num: int, device="cpu"):
    """1-based RotMat / RotMatInv [V, R]: view r turns every ring by r * n_theta / R
    angular steps (the shipped Factors/*/RotMat_full.csv are such permutations)."""
    if n_theta % rotate_num != 0:
        raise ValueError("n_theta must be divisible by rotate_num for cyclic rotation tables")
    step = n_theta // rotate_num
    V = n_r * n_theta
    j = torch.arange(V, device=device)
    ring, th = j // n_theta, j % n_theta
    rot = torch.empty((V, rotate_num), dtype=torch.int64, device=device)
    inv = torch.empty_like(rot)
    for r in range(rotate_num):
        rot[:, r] = ring * n_theta + (th + r * step) % n_theta + 1
        inv[:, r] = ring * n_theta + (th - r * step) % n_theta + 1
    return rot, inv


def cylinder_pixels(radius: float, n_phi: int, n_axial: int, axial_pitch: float, phi0: float = 0.0,
                    device="cpu") -> torch.Tensor:
    """Pixel centres [n_axial * n_phi, 3], azimuth fastest."""
    phi = phi0 + 2.0 * math.pi * (torch.arange(n_phi, dtype=torch.float64, device=device) + 0.5) / n_phi
    z = (torch.arange(n_axial, dtype=torch.float64, device=device) - (n_axial - 1) / 2.0) * axial_pitch
    zz, pp = torch.meshgrid(z, phi, indexing="ij")
    pos = torch.stack((radius * torch.cos(pp), radius * torch.sin(pp), zz), dim=-1)
    return pos.reshape(-1, 3)


def _disk_exit_path(c: torch.Tensor, d: torch.Tensor, obj_radius: float) -> torch.Tensor:
    """Length inside the object disk (xy-plane) from voxel c towards detector d."""
    v = d[..., :2] - c[..., :2]
    L = torch.sqrt((v * v).sum(-1)).clamp_min(1e-9)
    u = v / L.unsqueeze(-1)
    p = c[..., :2]
    b = (p * u).sum(-1)
    cc = (p * p).sum(-1) - obj_radius * obj_radius
    s = -b + torch.sqrt((b * b - cc).clamp_min(0.0))  # forward exit distance
    return torch.minimum(s.clamp_min(0.0), L)


def sc_system_matrix(coor: torch.Tensor, det_pos: torch.Tensor, pixel_area: float, obj_radius: float,
                     mu: float = 0.015, sigma: float = 0.2, generator: torch.Generator | None = None,
                     row_block: int = 1024, dtype=torch.float32) -> torch.Tensor:
    """Dense [n_det, V] SC matrix of the formula in the module docstring."""
    dev = coor.device
    n_det, V = det_pos.size(0), coor.size(0)
    out = torch.empty((n_det, V), dtype=dtype, device=dev)
    c = coor.to(torch.float32)
    for b0 in range(0, n_det, row_block):
        d = det_pos[b0:b0 + row_block].to(device=dev, dtype=torch.float32)
        vec = d.unsqueeze(1) - c.unsqueeze(0)                       # [b, V, 3]
        dist2 = (vec * vec).sum(-1).clamp_min(1e-6)
        dist = torch.sqrt(dist2)
        normal = -d / torch.sqrt((d[:, :2] ** 2).sum(-1, keepdim=True)).clamp_min(1e-9)
        normal[:, 2] = 0.0
        cos_inc = (-(vec * normal.unsqueeze(1)).sum(-1) / dist).clamp_min(0.0)
        path = _disk_exit_path(c.unsqueeze(0).expand_as(vec), d.unsqueeze(1).expand_as(vec), obj_radius)
        a = cos_inc * pixel_area / (4.0 * math.pi * dist2) * torch.exp(-mu * path)
        noise = torch.randn(a.shape, generator=generator, device=dev, dtype=torch.float32)
        out[b0:b0 + row_block] = (a * torch.exp(sigma * noise)).to(dtype)
    return out


def hot_rod_phantom(coor: torch.Tensor, disk_radius: float, contrast: float = 4.0) -> torch.Tensor:
    """Uniform disk (activity 1) with six hot rods (contrast:1) of radii 2..6 mm at
    half the disk radius."""
    x, y = coor[:, 0].double(), coor[:, 1].double()
    img = ((x * x + y * y) <= disk_radius ** 2).double()
    radii = torch.linspace(2.0, 6.0, 6, dtype=torch.float64)
    for k in range(6):
        ang = 2.0 * math.pi * k / 6.0
        cx, cy = 0.5 * disk_radius * math.cos(ang), 0.5 * disk_radius * math.sin(ang)
        rod = ((x - cx) ** 2 + (y - cy) ** 2) <= radii[k].item() ** 2
        img = torch.where(rod, torch.full_like(img, contrast), img)
    return img.to(torch.float32).unsqueeze(1)


def poisson_projection(A: torch.Tensor, x: torch.Tensor, total_counts: float,
                       generator: torch.Generator | None = None) -> torch.Tensor:
    """Poisson(A x) scaled so that the expected total is total_counts, as [B, 1]."""
    mean = torch.matmul(A.float(), x.float())
    mean = mean * (total_counts / mean.sum().clamp_min(1e-30))
    return torch.poisson(mean, generator=generator)


@dataclass
class ScProblem:
    grid: PolarGrid
    sysmat: torch.Tensor      # [B, V]
    proj: torch.Tensor        # [B, R]
    rotmat: torch.Tensor      # [V, R] int64 1-based
    rotmat_inv: torch.Tensor  # [V, R]
    s_map: torch.Tensor       # [V, 1]
    phantom: torch.Tensor     # [V, 1]


def sc_problem(n_r=40, n_theta=120, disk_radius=50.0, det_radius=120.0, n_phi=1024, n_axial=1,
               axial_pitch=1.0, views=10, flat=True, total_counts=1e6, seed=SEED, device="cpu",
               dtype=torch.float32) -> ScProblem:
    """Config-1 style SC problem (defaults: 40 x 120 grid, 1,024 pixels x 10 views)."""
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    grid = polar_grid(n_r, n_theta, disk_radius, device=device)
    pitch = 2.0 * math.pi * det_radius / n_phi
    area = pitch * axial_pitch
    if flat:
        blocks = []
        for v in range(views):
            pos = cylinder_pixels(det_radius, n_phi, n_axial, axial_pitch, phi0=2 * math.pi * v / views,
                                  device=device)
            blocks.append(sc_system_matrix(grid.coor, pos, area, disk_radius, generator=gen, dtype=dtype))
        A = torch.cat(blocks, dim=0)
        R = 1
        rot = torch.arange(1, grid.n_vox + 1, dtype=torch.int64, device=device).unsqueeze(1)
        inv = rot.clone()
    else:
        pos = cylinder_pixels(det_radius, n_phi, n_axial, axial_pitch, device=device)
        A = sc_system_matrix(grid.coor, pos, area, disk_radius, generator=gen, dtype=dtype)
        R = views
        rot, inv = cyclic_rotation_tables(n_r, n_theta, views, device=device)
    x = hot_rod_phantom(grid.coor, disk_radius).to(device)
    cols = []
    for r in range(R):
        xr = x[rot[:, r] - 1]
        cols.append(poisson_projection(A, xr, total_counts / R, generator=gen))
    proj = torch.cat(cols, dim=1)
    s = torch.zeros((grid.n_vox, 1), dtype=torch.float32, device=device)
    colsum = A.float().sum(dim=0, keepdim=True)
    for r in range(R):
        s += colsum[:, inv[:, r] - 1].transpose(0, 1)
    s = s / R
    return ScProblem(grid, A, proj, rot, inv, s, x)


# ----------------------------------------------------------------------------- Compton lists
def _kn_cos_theta(n, e0, generator, device):
    """Scatter-angle cosines from the Klein-Nishina distribution (rejection sampling)."""
    k = e0 / 0.511
    out = torch.empty(n, dtype=torch.float64, device=device)
    filled = 0
    while filled < n:
        m = 2 * (n - filled) + 1024
        c = torch.rand(m, generator=generator, device=device, dtype=torch.float64) * 2 - 1
        ratio = 1.0 / (1.0 + k * (1.0 - c))
        f = ratio * ratio * (ratio + 1.0 / ratio - (1.0 - c * c))   # (E'/E)^2 (E'/E + E/E' - sin^2)
        u = torch.rand(m, generator=generator, device=device, dtype=torch.float64) * 2.0
        acc = c[u < f]
        take = min(acc.numel(), n - filled)
        out[filled:filled + take] = acc[:take]
        filled += take
    return out


def compton_list(coor, activity, scat_pos, abs_radius, abs_n_phi, abs_n_axial, abs_pitch, e0, n_events, generator,
                 cp1_offset=0, cp2_offset=0, abs_phi0=0.0):
    """Forward-simulated two-interaction events (cp1, e1, cp2, e2) with 1-based ids.

    Source voxel ~ activity; first interaction at a uniformly chosen scatter pixel; scatter
    angle from Klein-Nishina around the source -> pixel direction, uniform azimuth; the
    scattered ray is intersected with the absorber cylinder (radius abs_radius, pixels of
    cylinder_pixels(abs_radius, abs_n_phi, abs_n_axial, abs_pitch, abs_phi0)); rays that miss
    its axial extent are dropped, so fewer than n_events may be returned. e1 = e0 - E'.
    Energy blur is left to the T builder (the reference smears in the builder)."""
    dev = coor.device
    n = int(n_events)
    src = coor[torch.multinomial(activity.flatten().double(), n, replacement=True, generator=generator)].double()
    i1 = torch.randint(scat_pos.size(0), (n,), generator=generator, device=dev)
    p1 = scat_pos[i1].double()
    d0 = p1 - src
    d0 = d0 / d0.norm(dim=1, keepdim=True)
    cos_t = _kn_cos_theta(n, e0, generator, dev)
    sin_t = torch.sqrt((1 - cos_t * cos_t).clamp_min(0))
    phi = torch.rand(n, generator=generator, device=dev, dtype=torch.float64) * (2 * math.pi)
    helper = torch.where(d0[:, 2:3].abs() < 0.9, torch.tensor([0.0, 0.0, 1.0], device=dev, dtype=torch.float64),
                         torch.tensor([1.0, 0.0, 0.0], device=dev, dtype=torch.float64))
    u = torch.linalg.cross(d0, helper)
    u = u / u.norm(dim=1, keepdim=True)
    w = torch.linalg.cross(d0, u)
    d1 = cos_t[:, None] * d0 + sin_t[:, None] * (torch.cos(phi)[:, None] * u + torch.sin(phi)[:, None] * w)
    # ray p1 + s d1 against the cylinder x^2 + y^2 = R^2 (outward root)
    a = d1[:, 0] ** 2 + d1[:, 1] ** 2
    b = 2 * (p1[:, 0] * d1[:, 0] + p1[:, 1] * d1[:, 1])
    c = p1[:, 0] ** 2 + p1[:, 1] ** 2 - abs_radius ** 2
    disc = (b * b - 4 * a * c).clamp_min(0)
    s = (-b + torch.sqrt(disc)) / (2 * a.clamp_min(1e-12))
    p2 = p1 + s[:, None] * d1
    half = abs_n_axial * abs_pitch / 2.0
    ok = (a > 1e-9) & (s > 0) & (p2[:, 2].abs() < half)
    ang = torch.remainder(torch.atan2(p2[:, 1], p2[:, 0]) - abs_phi0, 2 * math.pi)
    iphi = torch.clamp((ang / (2 * math.pi) * abs_n_phi).floor().long(), 0, abs_n_phi - 1)
    iz = torch.clamp(((p2[:, 2] + half) / abs_pitch).floor().long(), 0, abs_n_axial - 1)
    cp2 = iz * abs_n_phi + iphi
    e_sc = e0 / (1.0 + (e0 / 0.511) * (1.0 - cos_t))
    e1 = e0 - e_sc
    lst = torch.stack(((i1 + 1 + cp1_offset).double(), e1, (cp2 + 1 + cp2_offset).double(), e_sc), dim=1)
    return lst[ok].to(torch.float32)
