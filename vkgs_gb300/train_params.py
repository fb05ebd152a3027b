"""Raw per-splat parameters of the differentiable path, from 3DGS PLY rows.

The differentiable path takes the parameters before activation (what a trainer optimises):
means (N, 3), log-scales (N, 3), quaternions (N, 4) in (x, y, z, w) order, opacity logits (N,) and
degree-3 SH (N, 48) as FP32 in the reference's [channel][16 coefficients] layout (coefficient 0 =
f_dc_c, coefficient i + 1 = f_rest_{15 c + i}; parse_ply.comp:91-94, splat_load_thread.cc:114-135).
"""

from __future__ import annotations

import numpy as np

from . import synthetic as syn


def from_rows(rows: np.ndarray, properties=syn.PLY_PROPERTIES) -> dict:
    """numpy float32 arrays {means, log_scales, quats, opacity_logits, sh} from PLY rows."""
    at = {name: i for i, name in enumerate(properties)}
    r = np.asarray(rows, np.float32)
    sh = np.zeros((r.shape[0], 3, 16), np.float32)
    for c in range(3):
        sh[:, c, 0] = r[:, at[f"f_dc_{c}"]]
        for i in range(15):
            sh[:, c, i + 1] = r[:, at[f"f_rest_{15 * c + i}"]]
    return dict(
        means=np.ascontiguousarray(r[:, [at["x"], at["y"], at["z"]]]),
        log_scales=np.ascontiguousarray(r[:, [at["scale_0"], at["scale_1"], at["scale_2"]]]),
        quats=np.ascontiguousarray(r[:, [at["rot_1"], at["rot_2"], at["rot_3"], at["rot_0"]]]),
        opacity_logits=np.ascontiguousarray(r[:, at["opacity"]]),
        sh=np.ascontiguousarray(sh.reshape(-1, 48)),
    )
