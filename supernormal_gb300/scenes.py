"""Synthetic multi-view normal-map scenes with analytic SDF ground truth.

Stand-in for the DiLiGenT-MV data SuperNormal trains on (models/dataset_loader.py),
which is not shipped here: an analytic SDF (sphere, displaced torus, unions of
spheres / tori / boxes) is sphere-traced from pinhole cameras on a ring to give
world-space normal maps and masks.  Cameras follow the dataset's conventions
(OpenCV axes: x right, y down, z forward; pose = camera-to-world), rays are
``pose[:3,:3] @ normalize(K^-1 [x, y, 1])`` at integer pixel coordinates, the
marching-plane normal is the camera z axis and V^-1 = inv([d; right; down])
per pixel (models/dataset_loader.py:112-137, :223-277).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import torch
from torch import Tensor

__all__ = ["SDFScene", "sphere", "displaced_torus", "box", "union", "CameraRig", "ring_cameras",
           "SyntheticDataset", "random_scene"]


# ---------------------------------------------------------------------------
# analytic SDFs (torch, any device / dtype)
# ---------------------------------------------------------------------------
@dataclass
class SDFScene:
    """An analytic signed distance (approximate where displaced) with a
    Lipschitz bound used to keep sphere tracing conservative.  ``prims`` /
    ``disp`` describe the same scene to the device ground-truth renderer
    (``sn_scene_render_gt``): (kind, centre, size, amp, freq) per primitive
    and the union displacement (amp, freq); empty when the scene is not a
    plain union of at most four primitives."""

    fn: callable
    lipschitz: float = 1.0
    name: str = "scene"
    prims: tuple = ()
    disp: tuple = (0.0, 0.0)

    def descriptor(self):
        """The scene as an ``sn_scene_desc`` (None when it has no descriptor)."""
        from ._lib import SN_SCENE_MAX_PRIMS, SceneDesc

        if not self.prims or len(self.prims) > SN_SCENE_MAX_PRIMS:
            return None
        d = SceneDesc()
        d.n_prims = len(self.prims)
        for k, (kind, ctr, size, amp, freq) in enumerate(self.prims):
            p = d.prims[k]
            p.kind = kind
            for i in range(3):
                p.center[i] = float(ctr[i])
                p.size[i] = float(size[i])
            p.amp, p.freq = float(amp), float(freq)
        d.disp_amp, d.disp_freq = float(self.disp[0]), float(self.disp[1])
        d.lipschitz = float(self.lipschitz)
        return d

    def __call__(self, p: Tensor) -> Tensor:
        return self.fn(p)

    def normal(self, p: Tensor) -> Tensor:
        with torch.enable_grad():
            q = p.detach().requires_grad_(True)
            d = self.fn(q)
            (g,) = torch.autograd.grad(d.sum(), q)
        return torch.nn.functional.normalize(g, dim=-1)


def sphere(radius: float = 0.5, center=(0.0, 0.0, 0.0)) -> SDFScene:
    c = torch.tensor(center)

    def f(p):
        return torch.linalg.vector_norm(p - c.to(p), dim=-1) - radius

    return SDFScene(f, 1.0, f"sphere(r={radius})", prims=((0, tuple(center), (radius, 0.0, 0.0), 0.0, 0.0),))


def displaced_torus(R: float = 0.5, r: float = 0.2, amp: float = 0.02, freq: float = 20.0,
                    center=(0.0, 0.0, 0.0)) -> SDFScene:
    """Torus around the z axis with a radial displacement amp*sin(f*theta)*sin(f*phi)."""
    c = torch.tensor(center)

    def f(p):
        q = p - c.to(p)
        rxy = torch.sqrt(q[..., 0] ** 2 + q[..., 1] ** 2)
        ring = rxy - R
        d = torch.sqrt(ring ** 2 + q[..., 2] ** 2) - r
        if amp != 0.0:
            theta = torch.atan2(q[..., 1], q[..., 0])
            phi = torch.atan2(q[..., 2], ring)
            d = d - amp * torch.sin(freq * theta) * torch.sin(freq * phi)
        return d

    lip = 1.0 + abs(amp) * freq * (1.0 / max(R - r, 1e-3) + 1.0 / r)
    return SDFScene(f, lip, f"torus(R={R},r={r},amp={amp},freq={freq})",
                    prims=((1, tuple(center), (R, r, 0.0), amp, freq),))


def box(half=(0.3, 0.3, 0.3), center=(0.0, 0.0, 0.0)) -> SDFScene:
    h = torch.tensor(half)
    c = torch.tensor(center)

    def f(p):
        q = (p - c.to(p)).abs() - h.to(p)
        outside = torch.linalg.vector_norm(q.clamp_min(0.0), dim=-1)
        inside = q.amax(dim=-1).clamp_max(0.0)
        return outside + inside

    return SDFScene(f, 1.0, f"box({tuple(half)})", prims=((2, tuple(center), tuple(half), 0.0, 0.0),))


def union(*scenes: SDFScene, displacement: float = 0.0, freq: float = 20.0) -> SDFScene:
    def f(p):
        d = torch.stack([s(p) for s in scenes], dim=0).amin(dim=0)
        if displacement:
            d = d - displacement * torch.sin(freq * p[..., 0]) * torch.sin(freq * p[..., 1]) * \
                torch.sin(freq * p[..., 2])
        return d

    lip = max(s.lipschitz for s in scenes) + abs(displacement) * freq * math.sqrt(3.0)
    plain = all(s.prims and s.disp[0] == 0.0 for s in scenes)
    prims = tuple(p for s in scenes for p in s.prims) if plain else ()
    return SDFScene(f, lip, "union(" + ",".join(s.name for s in scenes) + ")", prims=prims,
                    disp=(displacement, freq) if displacement else (0.0, 0.0))


def random_scene(seed: int) -> SDFScene:
    """Seeded union of 1-3 spheres / tori / boxes inside the unit sphere with
    displacement amplitude in [0.005, 0.03]."""
    g = torch.Generator().manual_seed(seed)
    parts = []
    n = int(torch.randint(1, 4, (1,), generator=g))
    for _ in range(n):
        kind = int(torch.randint(0, 3, (1,), generator=g))
        ctr = ((torch.rand(3, generator=g) - 0.5) * 0.5).tolist()
        if kind == 0:
            parts.append(sphere(float(0.15 + 0.2 * torch.rand(1, generator=g)), ctr))
        elif kind == 1:
            parts.append(displaced_torus(0.3, 0.1, 0.0, 20.0, ctr))
        else:
            parts.append(box(tuple((0.1 + 0.15 * torch.rand(3, generator=g)).tolist()), ctr))
    amp = float(0.005 + 0.025 * torch.rand(1, generator=g))
    return union(*parts, displacement=amp)


# ---------------------------------------------------------------------------
# cameras
# ---------------------------------------------------------------------------
@dataclass
class CameraRig:
    poses: Tensor        # (n, 4, 4) camera-to-world
    intrinsics: Tensor   # (n, 4, 4)
    H: int
    W: int


def look_at(eye: Tensor, target: Tensor, up: Tensor) -> Tensor:
    z = torch.nn.functional.normalize(target - eye, dim=-1)          # forward
    x = torch.nn.functional.normalize(torch.linalg.cross(z, up), dim=-1)  # right
    y = torch.linalg.cross(z, x)                                      # down
    pose = torch.eye(4, dtype=eye.dtype)
    pose[:3, 0], pose[:3, 1], pose[:3, 2], pose[:3, 3] = x, y, z, eye
    return pose


def ring_cameras(n_views: int, H: int, W: int, radius: float = 3.0, elevation_deg: float = 0.0,
                 fov_deg: float = 40.0, dtype=torch.float64) -> CameraRig:
    """n_views pinhole cameras evenly spaced on a ring (axis z) looking at the origin."""
    poses, Ks = [], []
    f = 0.5 * W / math.tan(0.5 * math.radians(fov_deg))
    el = math.radians(elevation_deg)
    for i in range(n_views):
        az = 2.0 * math.pi * i / n_views
        eye = torch.tensor([radius * math.cos(el) * math.cos(az), radius * math.cos(el) * math.sin(az),
                            radius * math.sin(el)], dtype=dtype)
        poses.append(look_at(eye, torch.zeros(3, dtype=dtype), torch.tensor([0.0, 0.0, 1.0], dtype=dtype)))
        K = torch.eye(4, dtype=dtype)
        K[0, 0] = K[1, 1] = f
        K[0, 2], K[1, 2] = 0.5 * (W - 1), 0.5 * (H - 1)
        Ks.append(K)
    return CameraRig(torch.stack(poses), torch.stack(Ks), H, W)


# ---------------------------------------------------------------------------
# ground truth rendering
# ---------------------------------------------------------------------------
def pixel_rays(rig: CameraRig, view: int, px: Tensor, py: Tensor) -> Tensor:
    """World ray directions at integer pixel coordinates (float64)."""
    Kinv = inv3x3(rig.intrinsics[view, :3, :3]).to(px.device)
    p = torch.stack([px, py, torch.ones_like(px)], dim=-1).to(Kinv.dtype)
    v = p @ Kinv.T
    v = v / torch.linalg.vector_norm(v, dim=-1, keepdim=True)
    return v @ rig.poses[view, :3, :3].to(px.device).T


def view_rays(rig: CameraRig, view: int, device) -> tuple:
    """Ray directions (H, W, 3) and per-pixel V^-1 (H, W, 3, 3) of one view,
    float32, without ground truth (models/dataset_loader.py:112-137: V has
    rows d, camera right, camera down)."""
    H, W = rig.H, rig.W
    ys, xs = torch.meshgrid(torch.arange(H, device=device, dtype=torch.float64),
                            torch.arange(W, device=device, dtype=torch.float64), indexing="ij")
    d = pixel_rays(rig, view, xs, ys)
    right = rig.poses[view, :3, 0].to(device).expand_as(d)
    down = rig.poses[view, :3, 1].to(device).expand_as(d)
    V = torch.stack([d, right, down], dim=-2)
    return d.float(), inv3x3(V).float()


def sphere_trace(scene: SDFScene, o: Tensor, d: Tensor, near: Tensor, far: Tensor,
                 iters: int = 400, eps: float = 1e-6):
    t = near.clone()
    alive = torch.ones_like(t, dtype=torch.bool)
    hit = torch.zeros_like(alive)
    for _ in range(iters):
        p = o + d * t[..., None]
        s = scene(p)
        newly = alive & (s.abs() < eps)
        hit |= newly
        alive &= ~newly
        t = torch.where(alive, t + s / scene.lipschitz * 0.9, t)
        alive &= t < far
        if not alive.any():
            break
    return t, hit


def render_view_gt(scene: SDFScene, rig: CameraRig, view: int, xs: Tensor, ys: Tensor):
    """Ground-truth normals (N, 3) and hit mask of one view at pixel
    coordinates (xs, ys) with torch float64 ops (any device)."""
    d = pixel_rays(rig, view, xs, ys)
    o = rig.poses[view, :3, 3].to(xs.device).expand_as(d)
    near, far = _near_far(o, d)
    t, hit = sphere_trace(scene, o.reshape(-1, 3), d.reshape(-1, 3), near.reshape(-1), far.reshape(-1))
    pts = o.reshape(-1, 3) + d.reshape(-1, 3) * t[:, None]
    return scene.normal(pts) * hit[:, None], hit


@dataclass
class SyntheticDataset:
    """Views of an analytic scene with GT normals / masks, resident on
    `device`; gen_random_patches mirrors the reference sampler.  On a GPU the
    ground truth of a scene with a descriptor comes from one
    ``sn_scene_render_gt`` launch (double sphere tracing); otherwise from
    the torch float64 path (``render_view_gt``).  On a GPU the
    patches' rays and V^-1 are formed per pixel by `sn_gen_patches`, so no
    per-pixel (H, W, 3) ray or (H, W, 3, 3) V^-1 table is kept (48 B per
    pixel); `rays_all` / `V_inverse_all` build those tables on first use."""

    scene: SDFScene
    rig: CameraRig
    device: torch.device
    normals: Tensor = field(init=False)      # (n, H, W, 3) float32
    masks: Tensor = field(init=False)        # (n, H, W) float32
    kinv: Tensor = field(init=False)         # (n, 3, 3) float64 K^-1
    pose34: Tensor = field(init=False)       # (n, 3, 4) float64 [R | t]

    def __post_init__(self):
        n, H, W = self.rig.poses.shape[0], self.rig.H, self.rig.W
        dev = self.device
        self.pose_all = self.rig.poses.to(dev).float()
        self.intrinsics_all = self.rig.intrinsics.to(dev).float()
        self.kinv = inv3x3(self.rig.intrinsics[:, :3, :3].double()).to(dev).contiguous()
        self.pose34 = self.rig.poses[:, :3, :4].double().to(dev).contiguous()
        self.n_images, self.H, self.W = n, H, W
        self._tables = None
        desc = self.scene.descriptor()
        if dev.type == "cuda" and desc is not None:
            # one launch for every view (sn_scene_render_gt: double sphere tracing)
            from ._lib import call, stream_handle

            self.normals = torch.empty((n, H, W, 3), device=dev)
            self.masks = torch.empty((n, H, W), device=dev)
            call("sn_scene_render_gt", C.byref(desc), n, H, W, self.kinv, self.pose34, 400, 1e-6,
                 self.normals, self.masks, stream_handle())
            return
        ys, xs = torch.meshgrid(torch.arange(H, device=dev, dtype=torch.float64),
                                torch.arange(W, device=dev, dtype=torch.float64), indexing="ij")
        normals, masks = [], []
        for v in range(n):
            nrm, hit = render_view_gt(self.scene, self.rig, v, xs, ys)
            normals.append(nrm.reshape(H, W, 3).float())
            masks.append(hit.reshape(H, W).float())
        self.normals = torch.stack(normals)
        self.masks = torch.stack(masks)

    def _build_tables(self):
        if self._tables is None:
            views = [view_rays(self.rig, v, self.device) for v in range(self.n_images)]
            self._tables = (torch.stack([d for d, _ in views]), torch.stack([vi for _, vi in views]))
        return self._tables

    @property
    def rays_all(self) -> Tensor:
        """(n, H, W, 3) float32 ray directions, built on first use."""
        return self._build_tables()[0]

    @property
    def V_inverse_all(self) -> Tensor:
        """(n, H, W, 3, 3) float32 V^-1 (models/dataset_loader.py:112-137), built on first use."""
        return self._build_tables()[1]

    def gen_random_patches(self, num_patch: int, patch_H: int = 3, patch_W: int = 3,
                           generator: Optional[torch.Generator] = None):
        """Random patches from random views (models/dataset_loader.py:223-277)."""
        dev = self.device
        g = generator
        cx = torch.randint(patch_W // 2, self.W - 1 - patch_W // 2, (num_patch,), device=dev, generator=g)
        cy = torch.randint(patch_H // 2, self.H - 1 - patch_H // 2, (num_patch,), device=dev, generator=g)
        img = torch.randint(0, self.n_images, (num_patch,), device=dev, generator=g)
        if self.device.type == "cuda":
            from ._lib import call, stream_handle

            shp = (num_patch, patch_H, patch_W)
            rays_o = torch.empty(shp + (3,), device=dev)
            rays_d = torch.empty(shp + (3,), device=dev)
            plane_n = torch.empty((num_patch, 3), device=dev)
            vinv = torch.empty(shp + (3, 3), device=dev)
            normal = torch.empty(shp + (3,), device=dev)
            mask = torch.empty(shp + (1,), device=dev)
            call("sn_gen_patches", num_patch, patch_H, patch_W, cx.int(), cy.int(), img.int(), self.n_images,
                 self.H, self.W, self.kinv, self.pose34, self.normals, self.masks, rays_o, rays_d, plane_n,
                 vinv, normal, mask, stream_handle())
            return rays_o, rays_d, plane_n, vinv, normal, mask
        ox = torch.arange(-(patch_W // 2), patch_W // 2 + 1, device=dev)
        oy = torch.arange(-(patch_H // 2), patch_H // 2 + 1, device=dev)
        px = cx[:, None, None] + ox[None, None, :].expand(1, patch_H, patch_W)
        py = cy[:, None, None] + oy[None, :, None].expand(1, patch_H, patch_W)
        iv = img[:, None, None].expand_as(px)
        normal = self.normals[iv, py, px]
        vinv = self.V_inverse_all[iv, py, px]
        mask = self.masks[iv, py, px].unsqueeze(-1)
        rays_d = self.rays_all[iv, py, px]
        rays_o = self.pose_all[img, None, None, :3, 3].expand(rays_d.shape)
        plane_n = self.pose_all[img, :3, 2]
        return (rays_o.contiguous(), rays_d.contiguous(), plane_n.contiguous(), vinv.contiguous(),
                normal.contiguous(), mask.contiguous())


def sample_patches(scene: SDFScene, rig: CameraRig, num_patch: int, patch_H: int = 3, patch_W: int = 3,
                   generator: Optional[torch.Generator] = None, device="cpu"):
    """gen_random_patches for just the sampled pixels (sphere-traced on demand), so a
    host-only consumer needs no full-view ground truth.  Same outputs and layout."""
    g = generator
    H, W, n = rig.H, rig.W, rig.poses.shape[0]
    cx = torch.randint(patch_W // 2, W - 1 - patch_W // 2, (num_patch,), generator=g)
    cy = torch.randint(patch_H // 2, H - 1 - patch_H // 2, (num_patch,), generator=g)
    img = torch.randint(0, n, (num_patch,), generator=g)
    ox = torch.arange(-(patch_W // 2), patch_W // 2 + 1)
    oy = torch.arange(-(patch_H // 2), patch_H // 2 + 1)
    px = (cx[:, None, None] + ox[None, None, :]).expand(num_patch, patch_H, patch_W).double()
    py = (cy[:, None, None] + oy[None, :, None]).expand(num_patch, patch_H, patch_W).double()
    rays = torch.empty((num_patch, patch_H, patch_W, 3), dtype=torch.float64)
    for v in img.unique().tolist():
        sel = img == v
        rays[sel] = pixel_rays(rig, v, px[sel], py[sel])
    o = rig.poses[img, :3, 3][:, None, None, :].expand_as(rays)
    near, far = _near_far(o, rays)
    t, hit = sphere_trace(scene, o.reshape(-1, 3), rays.reshape(-1, 3), near.reshape(-1), far.reshape(-1))
    pts = o.reshape(-1, 3) + rays.reshape(-1, 3) * t[:, None]
    normal = (scene.normal(pts) * hit[:, None]).reshape(num_patch, patch_H, patch_W, 3)
    mask = hit.reshape(num_patch, patch_H, patch_W, 1).double()
    right = rig.poses[img, :3, 0][:, None, None, :].expand_as(rays)
    down = rig.poses[img, :3, 1][:, None, None, :].expand_as(rays)
    vinv = inv3x3(torch.stack([rays, right, down], dim=-2))
    plane_n = rig.poses[img, :3, 2]
    f = lambda a: a.float().contiguous().to(device)
    return f(o), f(rays), f(plane_n), f(vinv), f(normal), f(mask)


def inv3x3(M: Tensor) -> Tensor:
    """Inverse of (..., 3, 3) matrices by the adjugate (rows r0, r1, r2:
    inverse columns are r1 x r2, r2 x r0, r0 x r1 over the determinant)."""
    r0, r1, r2 = M[..., 0, :], M[..., 1, :], M[..., 2, :]
    c0 = torch.linalg.cross(r1, r2)
    c1 = torch.linalg.cross(r2, r0)
    c2 = torch.linalg.cross(r0, r1)
    det = (r0 * c0).sum(-1, keepdim=True)
    return torch.stack([c0 / det, c1 / det, c2 / det], dim=-1)


def _near_far(o: Tensor, d: Tensor):
    a = (d * d).sum(-1)
    b = 2.0 * (o * d).sum(-1)
    c = (o * o).sum(-1) - 1.0
    disc = (b * b - 4 * a * c).clamp_min(0.0)
    mid = -0.5 * b / a
    return mid - disc.sqrt() / (2 * a), mid + disc.sqrt() / (2 * a)
