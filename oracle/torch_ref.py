"""FP64 torch restatement of the differentiable path (TEST INFRASTRUCTURE -- the gradient oracle).

Forward from raw per-splat parameters to the RGBA image, in float64 with autograd, following the same
reference formulas as the scalar C restatement (``oracle/cpu_ref.c``):

* activation, parse_ply.comp:34-97 -- s = exp(log_s); q = quat / |quat| in (x, y, z, w) order;
  cov3d = R(q) diag(s^2) R(q)^T; opacity = sigmoid(logit); SH used as given (FP32 coefficients);
* projection.comp:80-179 -- pv = V M pos; cov = (V3 M3) cov3d (V3 M3)^T; J rows (-1/z, 0, x/z^2),
  (0, -1/z, y/z^2); cov2d = P2 (J cov J^T)_2x2 P2 + diag(1/W^2, 1/H^2); ndc = (P pv).xy / w;
  colour = max(SH . basis(normalize(pos - M^-1 eye)) + 0.5, 0), clamped to 1 by the UNORM target;
* splat.vert / splat.frag -- coverage |(rot_scale^-1 (pixel - c))_i| <= 3 (a mask: no gradient),
  alpha = o exp(-1/2 d^T cov2d^-1 d) (rot_scale rot_scale^T = cov2d);
* blend, engine.cc:281-300 -- front to back in the given sorted order: RGB = sum a_i rgb_i T_i,
  A = sum a_i^2 T_i + T_end, from (0, 0, 0, 1).

The visible set and the draw order are inputs (the bit-exact FP32 ones from the CUDA path or the C
oracle), so the oracle differentiates exactly the frame the renderer drew.  Nothing in the product
imports this module.
"""

from __future__ import annotations

import math

import torch

C0 = 0.28209479177387814
C1 = 0.4886025119029199
C20, C21, C22 = 1.0925484305920792, 0.31539156525252005, 0.5462742152960396
C30, C31, C32, C33, C34 = 0.5900435899266435, 2.890611442640554, 0.4570457994644658, 0.3731763325901154, 1.445305721320277


def rotation(q):
    """(n, 4) unit quaternions (x, y, z, w) -> (n, 3, 3) rotation matrices (row, column)."""
    x, y, z, w = q.unbind(-1)
    xx, yy, zz = x * x, y * y, z * z
    xy, xz, yz = x * y, x * z, y * z
    wx, wy, wz = w * x, w * y, w * z
    r = torch.stack([
        1 - 2 * (yy + zz), 2 * (xy - wz), 2 * (xz + wy),
        2 * (xy + wz), 1 - 2 * (xx + zz), 2 * (yz - wx),
        2 * (xz - wy), 2 * (yz + wx), 1 - 2 * (xx + yy)], -1)
    return r.reshape(q.shape[:-1] + (3, 3))


def sh_basis(d):
    """(n, 3) unit directions -> (n, 16) degree-3 basis in the reference's coefficient order."""
    x, y, z = d.unbind(-1)
    xx, yy, zz = x * x, y * y, z * z
    xy, yz, xz = x * y, y * z, x * z
    return torch.stack([
        torch.full_like(x, C0), -C1 * y, C1 * z, -C1 * x,
        C20 * xy, -C20 * yz, C21 * (2 * zz - xx - yy), -C20 * xz,
        C22 * (xx - yy), -C30 * y * (3 * xx - yy), C31 * xy * z, -C32 * y * (4 * zz - xx - yy),
        C33 * z * (2 * zz - 3 * xx - 3 * yy), -C32 * x * (4 * zz - xx - yy), C34 * z * (xx - yy),
        -C30 * x * (xx - 3 * yy)], -1)


def mat(m16):
    """Column-major 16 floats -> (4, 4) float64 matrix in (row, column) indexing."""
    return torch.as_tensor(m16, dtype=torch.float64).reshape(4, 4).T


def project(means, log_scales, quats, opacity_logits, sh, cam):
    """Per-splat centre (n, 2), cov2d entries (n, 3) = (a, b, c), colour (n, 3), opacity (n,), depth (n,)."""
    P, V, M = mat(cam["projection"]), mat(cam["view"]), mat(cam["model"])
    W, H = float(cam["width"]), float(cam["height"])
    s = torch.exp(log_scales)
    q = quats / quats.norm(dim=-1, keepdim=True)
    R = rotation(q)
    cov3d = R @ torch.diag_embed(s * s) @ R.transpose(-1, -2)
    o = torch.sigmoid(opacity_logits)
    ones = torch.ones_like(means[:, :1])
    ph = torch.cat([means, ones], -1)
    pv = ph @ (V @ M).T  # (n, 4)
    A = (V[:3, :3] @ M[:3, :3])
    cov = A @ cov3d @ A.T
    x, y, z = pv[:, 0], pv[:, 1], pv[:, 2]
    zero = torch.zeros_like(z)
    J = torch.stack([torch.stack([-1 / z, zero, x / z / z], -1), torch.stack([zero, -1 / z, y / z / z], -1)], -2)
    c2 = J @ cov @ J.transpose(-1, -2)
    P2 = P[:2, :2]
    cov2d = P2 @ c2 @ P2
    a = cov2d[:, 0, 0] + 1.0 / W / W
    b = cov2d[:, 1, 1] + 1.0 / H / H
    c = cov2d[:, 1, 0]
    pc = pv @ P.T
    centre = pc[:, :2] / pc[:, 3:4]
    depth = pc[:, 2] / pc[:, 3]
    eye = torch.as_tensor(cam["eye"], dtype=torch.float64)
    cam_m = torch.linalg.solve(M, torch.cat([eye, eye.new_ones(1)]))
    cam_m = cam_m[:3] / cam_m[3]
    d = means - cam_m
    d = d / d.norm(dim=-1, keepdim=True)
    basis = sh_basis(d)  # (n, 16)
    col = torch.einsum("nk,nck->nc", basis, sh.reshape(-1, 3, 16)) + 0.5
    col = torch.clamp(col, min=0.0, max=1.0)
    return centre, torch.stack([a, b, c], -1), col, o, depth


def rot_scale_inverse(cov2d):
    """Rows (m00, m01), (m10, m11) of rot_scale^-1 by the reference's eigen decomposition (no gradient)."""
    with torch.no_grad():
        a, b, c = cov2d.unbind(-1)
        D = torch.sqrt((a - b) ** 2 + 4 * c * c)
        s0 = torch.sqrt(0.5 * (a + b + D))
        s1 = torch.sqrt(0.5 * (a + b - D))
        th = 0.5 * torch.atan2(2 * c / D, (a - b) / D)
        ct, st = torch.cos(th), torch.sin(th)
        m = torch.stack([ct / s0, st / s0, -st / s1, ct / s1], -1)
        drawn = (s1 > 0) & torch.isfinite(m).all(-1)
        return m, drawn


def render(means, log_scales, quats, opacity_logits, sh, cam, order, chunk=4096, mask_records=None, window=None):
    """RGBA (H, W, 4) float64 for splats `order` (sorted draw order, far to near), autograd-capable.

    mask_records: optional (V, 16) FP32 raster records of the same splats in the same order (the C
    oracle's): coverage is then decided in FP32 with the renderer's rounding (dx = px - cx,
    u = m00 dx + m01 dy, one rounding per operation), so both sides blend the same (pixel, splat) set.
    window: optional pixel rectangle (x0, x1, y0, y1), half-open: only those pixels are drawn and the
    result is (y1 - y0, x1 - x0, 4) -- every pixel's value is the same as in the whole image."""
    W, H = int(cam["width"]), int(cam["height"])
    x0, x1, y0, y1 = (0, W, 0, H) if window is None else (int(v) for v in window)
    idx = torch.as_tensor(order, dtype=torch.long)
    centre, cov2d, col, o, depth = project(means[idx], log_scales[idx], quats[idx], opacity_logits[idx], sh[idx], cam)
    m, drawn = rot_scale_inverse(cov2d)
    keep = drawn & (depth >= 0) & (depth < 1)
    rec = None
    if mask_records is not None:
        rec = torch.as_tensor(mask_records, dtype=torch.float32)
        keep = rec[:, 12] >= 0
    det = cov2d[:, 0] * cov2d[:, 1] - cov2d[:, 2] ** 2
    conic = torch.stack([cov2d[:, 1] / det, cov2d[:, 0] / det, -cov2d[:, 2] / det], -1)  # (A, B, C) of the inverse
    # nearest first for the front-to-back sum
    centre, conic, col, o, m, keep = (t.flip(0) for t in (centre, conic, col, o, m, keep))
    if rec is not None:
        rec = rec.flip(0)
    ys, xs = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64), torch.arange(x0, x1, dtype=torch.float64),
                            indexing="ij")
    px = ((2 * xs + 1) / W - 1).reshape(-1)
    py = ((2 * ys + 1) / H - 1).reshape(-1)
    px32 = ((2 * xs.float() + 1) / torch.tensor(float(W), dtype=torch.float32) - 1).reshape(-1)
    py32 = ((2 * ys.float() + 1) / torch.tensor(float(H), dtype=torch.float32) - 1).reshape(-1)
    out = []
    for s0 in range(0, px.shape[0], chunk):
        dx = px[None, s0:s0 + chunk] - centre[:, :1]
        dy = py[None, s0:s0 + chunk] - centre[:, 1:2]
        with torch.no_grad():
            if rec is None:
                u = m[:, 0:1] * dx + m[:, 1:2] * dy
                v = m[:, 2:3] * dx + m[:, 3:4] * dy
            else:
                dx32 = px32[None, s0:s0 + chunk] - rec[:, 0:1]
                dy32 = py32[None, s0:s0 + chunk] - rec[:, 1:2]
                u = rec[:, 2:3] * dx32 + rec[:, 3:4] * dy32
                v = rec[:, 4:5] * dx32 + rec[:, 5:6] * dy32
            cov = (u.abs() <= 3) & (v.abs() <= 3) & keep[:, None]
        qf = conic[:, 0:1] * dx * dx + 2 * conic[:, 2:3] * dx * dy + conic[:, 1:2] * dy * dy
        a = torch.where(cov, o[:, None] * torch.exp(-0.5 * qf), torch.zeros_like(qf))
        T = torch.cumprod(torch.cat([torch.ones_like(a[:1]), 1 - a], 0), 0)  # T[i] before splat i; T[-1] = T_end
        w = a * T[:-1]
        rgb = (w[:, :, None] * col[:, None, :]).sum(0)
        alpha = (w * a).sum(0) + T[-1]
        out.append(torch.cat([rgb, alpha[:, None]], -1))
    return torch.cat(out, 0).reshape(y1 - y0, x1 - x0, 4)


def camera_dict(oracle_cam: dict) -> dict:
    """The tests' camera dict (projection/view/model column-major, eye, width, height)."""
    return {k: oracle_cam[k] for k in ("projection", "view", "model", "eye", "width", "height")}


def central_difference(f, x: torch.Tensor, index, h: float = 1e-6) -> float:
    """d f / d x[index] by FP64 central differences."""
    with torch.no_grad():
        old = x[index].item()
        x[index] = old + h
        fp = f().item()
        x[index] = old - h
        fm = f().item()
        x[index] = old
    return (fp - fm) / (2 * h)


__all__ = ["render", "project", "rotation", "sh_basis", "central_difference", "camera_dict", "math"]
