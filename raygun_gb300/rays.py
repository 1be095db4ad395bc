"""Ray sets built on the device for the closest-hit queries of the benchmark and of profiling runs.

camera_rays_device: the pixel-centre camera rays of raygen.h:84-90.
first_bounce_secondary: the GENERIC reflection / refraction rays that closesthit.rchit:206-250 issues
at the hits of those camera rays, the incoherent secondary rays whose closest-hit throughput the
benchmark reports.
"""
from __future__ import annotations

import numpy as np


def camera_rays_device(ubo, width, height, dev):
    """Pixel-centre camera rays of raygen.h:84-90 (origin, tmin 0.001, direction, tmax 1e4) for a
    width x height image, on the device: n x 8 float32."""
    import torch
    u = ubo[0] if ubo.shape else ubo
    vi = torch.tensor(u["viewInverse"].reshape(4, 4), dtype=torch.float32, device=dev)  # [col][row]
    pi = torch.tensor(u["projInverse"].reshape(4, 4), dtype=torch.float32, device=dev)
    ys, xs = torch.meshgrid(torch.arange(height, device=dev, dtype=torch.float32),
                            torch.arange(width, device=dev, dtype=torch.float32), indexing="ij")
    d = torch.stack([(xs + 0.5) / width * 2 - 1, (ys + 0.5) / height * 2 - 1, torch.ones_like(xs), torch.ones_like(xs)], -1)
    t = (d.reshape(-1, 4) @ pi)[:, :3]
    t = t / t.norm(dim=1, keepdim=True)
    dirs = t @ vi[:3, :3]
    rays = torch.zeros(len(dirs), 8, device=dev)
    rays[:, :3] = vi[3, :3]
    rays[:, 3], rays[:, 7] = 0.001, 10000.0
    rays[:, 4:7] = dirs
    return rays


def first_bounce_secondary(ctx, sc, instances, dev, width, height):
    """The frame's first-bounce GENERIC secondary rays (closesthit.rchit:206-250): camera rays at
    width x height pixel centres traced on the GPU, then at every hit the reflection ray (material
    reflectivity > 0) and the refraction ray (transparency > 0, front face eta = 1/ior, back face eta =
    ior), from the hit point with tmin 0.01, tmax 1000, along the shading normal (object-to-world
    3x3 times the interpolated vertex normal, flipped toward the ray).  Total internal reflection
    (a zero direction) traverses nothing and is left out.  The grid effect's per-point material
    changes are not applied.  Returns n x 8 float32 on the device."""
    import torch
    cam = camera_rays_device(sc.ubo, width, height, dev).contiguous()
    n = len(cam)
    tuv = torch.empty(n, 3, device=dev)
    ids = torch.empty(n, 2, dtype=torch.int32, device=dev)
    if torch.device(dev).type == "cuda":
        torch.cuda.synchronize(dev)
    ctx.trace_rays_device(cam.data_ptr(), n, tuv.data_ptr(), ids.data_ptr())
    ctx.synchronize()
    inst_id = ids[:, 0].to(torch.int64) & 0xFFFFFFFF
    hit = inst_id != 0xFFFFFFFF
    cam, tuv, inst_id, prim = cam[hit], tuv[hit], inst_id[hit], ids[hit, 1].to(torch.int64) & 0xFFFFFFFF
    inst = instances
    xf = torch.tensor(inst["transform"], dtype=torch.float32, device=dev)[inst_id]            # (m, 3, 4)
    voff = torch.tensor(inst["vertexBufferOffset"].astype(np.int64), device=dev)[inst_id]
    ioff = torch.tensor(inst["indexBufferOffset"].astype(np.int64), device=dev)[inst_id]
    moff = torch.tensor(inst["materialBufferOffset"].astype(np.int64), device=dev)[inst_id]
    idx = torch.tensor(sc.indices.astype(np.int64), device=dev)
    vn = torch.tensor(sc.vertices["normal"], dtype=torch.float32, device=dev)
    vmat = torch.tensor(sc.vertices["matIndex"].astype(np.int64), device=dev)
    tri = torch.stack([idx[ioff + 3 * prim + k] for k in range(3)], 1) + voff[:, None]
    u, v = tuv[:, 1:2], tuv[:, 2:3]
    nrm = (1 - u - v) * vn[tri[:, 0]] + u * vn[tri[:, 1]] + v * vn[tri[:, 2]]
    nrm = torch.einsum("mij,mj->mi", xf[:, :, :3], nrm)
    nrm = nrm / nrm.norm(dim=1, keepdim=True)
    mats = sc.materials
    mi = moff + vmat[tri[:, 0]]
    refl = torch.tensor(mats["reflectivity"], dtype=torch.float32, device=dev)[mi]
    trans = torch.tensor(mats["transparency"], dtype=torch.float32, device=dev)[mi]
    ior = torch.tensor(mats["ior"], dtype=torch.float32, device=dev)[mi]
    o, d = cam[:, :3], cam[:, 4:7]
    p = o + d * tuv[:, :1]
    front = (-(d * nrm).sum(1)) > 0
    nrm = torch.where(front[:, None], nrm, -nrm)
    dn = (d * nrm).sum(1, keepdim=True)
    r_dir = d - 2 * dn * nrm
    eta = torch.where(front, 1.0 / ior, ior)[:, None]
    k = 1 - eta * eta * (1 - dn * dn)
    t_dir = torch.where(k >= 0, eta * d - (eta * dn + torch.sqrt(k.clamp_min(0))) * nrm, torch.zeros_like(d))
    out = []
    for sel, dd in ((refl > 0, r_dir), ((trans > 0) & (t_dir.abs().sum(1) > 0), t_dir)):
        r = torch.zeros(int(sel.sum()), 8, device=dev)
        r[:, :3], r[:, 3], r[:, 4:7], r[:, 7] = p[sel], 0.01, dd[sel], 1000.0
        out.append(r)
    return torch.cat(out).contiguous()
