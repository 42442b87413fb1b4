"""Parity protocol for the bake (shared by the GPU tests and the smoke check).

The device traces in FP32, the oracle in FP64.  Per-ray decisions (which
triangle is hit, whether the shadow ray is blocked) may legitimately differ
only where FP32 cannot decide: rays passing within EDGE_TOL of a triangle
edge, hits within EDGE_TOL of the ray interval's end, near-ties between two
triangles.  Everything else must agree.  The SH comparison then replays the
oracle with the device's decisions, so shading and projection are checked to
SH_TOL independently of those edge cases, and the direct comparison counts
the probes that edge rays pushed past SH_TOL.
"""
from __future__ import annotations

import numpy as np

EDGE_TOL = 1e-6      # world units, hit-ID tolerance from the specification
SHADOW_TOL = 1e-5    # shadow-ray margin (the hit point itself moves by FP32 rounding)
SH_TOL = 1e-4        # relative L2 per probe


def per_probe_rel(a, b):
    a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
    b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    return np.where(den > 0, num / np.maximum(den, 1e-300), num)


def classify(orc, probes, dirs32, sun, gpu_hit, gpu_vis, o_hit, o_vis, o_edge, tmin=1e-3, tmax=1e4, bias=5e-3,
             light=None):
    """Returns counts of explained / unexplained decision mismatches.  With
    `light` the shadow rays are the reference shading's (the winding normal,
    toward the point light, ending at it); else the sun's."""
    res = {"rays": int(gpu_hit.size), "hit_mismatch": 0, "hit_explained": 0, "shadow_mismatch": 0,
           "shadow_explained": 0, "unexplained": []}
    sunv = np.asarray(sun, np.float64)
    sunv = sunv / np.linalg.norm(sunv)
    for p, s in np.argwhere(gpu_hit != o_hit):
        res["hit_mismatch"] += 1
        o = probes[p].astype(np.float64)
        d = dirs32[s].astype(np.float64)
        eo = abs(o_edge[p, s]) if o_hit[p, s] >= 0 else np.inf
        eg, tg = np.inf, None
        if gpu_hit[p, s] >= 0:
            r = orc.ray_tri(o, d, gpu_hit[p, s])
            if r is not None:
                tg, eg = r[0], abs(r[3])
        t_o = orc.ray_tri(o, d, o_hit[p, s])[0] if o_hit[p, s] >= 0 else None
        near_tmin = (tg is not None and abs(tg - tmin) < EDGE_TOL) or (t_o is not None and abs(t_o - tmin) < EDGE_TOL)
        tie = tg is not None and t_o is not None and abs(tg - t_o) < EDGE_TOL * max(1.0, abs(t_o))
        if min(eo, eg) < EDGE_TOL or near_tmin or tie:
            res["hit_explained"] += 1
        else:
            res["unexplained"].append(("hit", int(p), int(s), int(o_hit[p, s]), int(gpu_hit[p, s]), eo, eg))
    same = (gpu_hit == o_hit) & (gpu_hit >= 0)
    for p, s in np.argwhere(same & (gpu_vis != o_vis)):
        res["shadow_mismatch"] += 1
        o = probes[p].astype(np.float64)
        d = dirs32[s].astype(np.float64)
        t, b1, b2, _ = orc.ray_tri(o, d, o_hit[p, s])
        P = o + t * d
        tri = orc.idx[o_hit[p, s]]
        v = orc.pos[tri].astype(np.float64)
        n = np.cross(v[1] - v[0], v[2] - v[0])
        n /= np.linalg.norm(n)
        if light is None:
            if n @ d > 0:
                n = -n
            ndl = n @ sunv
            m = orc.shadow_margin(P + bias * n, sunv, 0.0, tmax)
            end_flip = False
        else:
            S = np.asarray(light, np.float64) - P
            ln = np.linalg.norm(S)
            Ld = S / ln
            ndl = n @ Ld
            m = orc.shadow_margin(P + bias * n, Ld, 0.0, ln)
            # a blocker at the light itself: the interval's end decides it
            lo = orc.shadow_margin(P + bias * n, Ld, 0.0, ln * (1 - SHADOW_TOL))
            hi = orc.shadow_margin(P + bias * n, Ld, 0.0, ln * (1 + SHADOW_TOL))
            end_flip = (lo >= 0) != (hi >= 0)
        if abs(m) < SHADOW_TOL or abs(ndl) < 1e-6 or end_flip:
            res["shadow_explained"] += 1
        else:
            res["unexplained"].append(("shadow", int(p), int(s), m))
    return res
