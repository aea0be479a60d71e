"""Classification of product results against the oracle.

TEST INFRASTRUCTURE ONLY: a checker that tests/, the smoke check and bench.py's
parity report call; the product never imports it.

Every ray's product result falls in exactly one class:

  identical  same hit/miss and primitive; with exact=True also the same t, u, v
             bits (hits) as the oracle
  tie        a different primitive at the same distance: exact=True the same f32
             t; exact=False the two triangles' FP64 distances within TIE_REL
  nan        the ray can meet a NaN distance under the reference's triangle
             formula (geometry/mod.rs:105-155 gives t = 0/0 for a zero-area
             triangle or a ray in a triangle's plane, and accepts it), so the
             reference's own result depends on its walk order
  edge       the point where the ray meets the plane of a triangle that either
             side reports lies, in FP64, within the reference formula's f32
             position error of that triangle's boundary: 32 * 2^-24 * distance
             / |cos theta| (the formula's t is a quotient that loses accuracy as
             the ray grazes the plane) plus 1e-4 of the triangle's smallest
             altitude
  other      none of these: a real difference

The reference keeps the last of equal-distance hits (inclusive `t <= far`,
geometry/mod.rs:133, and the unconditional overwrite of traverse_cpu.rs:177-184);
an ordered walk meets them in another order, hence the tie class. Shadow rays
(first hit ends the search) are compared on hit/miss only.
"""

from __future__ import annotations

import numpy as np

from . import orc

TIE_REL = 1e-6
CLASSES = ("identical", "tie", "nan", "edge", "other")
IDENTICAL, TIE, NAN, EDGE, OTHER = range(5)


def _fp64(S, rays, prim, geometry, instance):
    h = np.zeros(len(rays), orc.HIT_DTYPE)
    h["prim"] = prim
    h["geometry"] = geometry
    h["instance"] = instance
    return S.eval_fp64(np.ascontiguousarray(rays), h)


def _near_edge(S, rays, prim, geometry, instance):
    """True where a reported hit's point lies within the f32 position error
    bound of the reference's formula from the triangle's boundary (inside or
    outside): FP64 distance to the nearest edge line against
    32 * 2^-24 * distance / |cos theta| plus 1e-4 of the smallest altitude."""
    h = np.zeros(len(rays), orc.HIT_DTYPE)
    h["prim"] = prim
    h["geometry"] = geometry
    h["instance"] = instance
    m = S.edge_margin(np.ascontiguousarray(rays), h)
    return np.abs(m[:, 0]) <= m[:, 1]


def classify_hits(S, rays, got_prim, got_t, got_u, got_v, exp, got_instance=None, got_geometry=None, exact=True,
                  tlas_idx=None, tlas_uniform=0, ray_flags=0, cull_mask=0xFF, first_hit=False, threads=16):
    """Classes of product hits against oracle hits `exp` (orc.HIT_DTYPE) for the
    same rays. got_instance / got_geometry: the product's instance slot and
    geometry index per ray (None: taken equal to the oracle's, as in scenes of
    one instance and one geometry). first_hit: a search that ends at its first
    hit (compared on hit/miss only). Returns an int8 class per ray."""
    n = len(rays)
    cls = np.zeros(n, np.int8)
    if n == 0:
        return cls
    e_prim = exp["prim"]
    gh, eh = got_prim != orc.MISS, e_prim != orc.MISS
    g_inst = exp["instance"] if got_instance is None else got_instance
    g_geom = exp["geometry"] if got_geometry is None else got_geometry
    if first_hit:
        identical = gh == eh
    else:
        same = (got_prim == e_prim) & ((~eh) | ((g_inst == exp["instance"]) & (g_geom == exp["geometry"])))
        if exact:
            bits = lambda a: np.ascontiguousarray(a, np.float32).view(np.uint32)  # noqa: E731
            same_val = (bits(got_t) == bits(exp["t"])) & (bits(got_u) == bits(exp["u"])) & (bits(got_v) == bits(exp["v"]))
            identical = same & ((~eh) | same_val)
        else:
            identical = same
    mism = np.nonzero(~identical)[0]
    if mism.size == 0:
        return cls
    r = np.ascontiguousarray(rays[mism])
    both = gh[mism] & eh[mism] & (not first_hit)
    if exact:
        tie = both & (np.asarray(got_t)[mism] == exp["t"][mism])
    else:
        tie = np.zeros(mism.size, bool)
    if first_hit:  # a first hit can be any triangle in range: no FP64 triangle to evaluate
        f_got = f_exp = np.full((mism.size, 3), np.nan)
    else:
        f_got = _fp64(S, r, np.where(gh[mism], got_prim[mism], orc.MISS), g_geom[mism], g_inst[mism])
        f_exp = _fp64(S, r, e_prim[mism], exp["geometry"][mism], exp["instance"][mism])
    if not exact:
        tg, te = f_got[:, 0], f_exp[:, 0]
        tie = both & (np.abs(tg - te) <= TIE_REL * np.maximum(np.abs(tg), np.abs(te)))
    ti = None if tlas_idx is None else np.ascontiguousarray(np.asarray(tlas_idx)[mism])
    nan = S.nan_exposure(r, tlas_idx=ti, tlas_uniform=tlas_uniform, ray_flags=ray_flags, cull_mask=cull_mask,
                         threads=threads)
    if first_hit:
        edge = np.zeros(mism.size, bool)
    else:
        edge = ((gh[mism] & _near_edge(S, r, np.where(gh[mism], got_prim[mism], orc.MISS), g_geom[mism], g_inst[mism]))
                | (eh[mism] & _near_edge(S, r, e_prim[mism], exp["geometry"][mism], exp["instance"][mism])))
    c = np.full(mism.size, OTHER, np.int8)
    c[edge] = EDGE
    c[nan] = NAN
    c[tie] = TIE
    cls[mism] = c
    return cls


def counts(cls) -> dict:
    out = {name: int((cls == k).sum()) for k, name in enumerate(CLASSES)}
    out["n"] = int(cls.size)
    return out


def classify_trace(S, rays, got, got_ext, exp, exact=True, **kw) -> tuple[np.ndarray, dict]:
    """rdn_trace results: got = hits (structured t, u, v, prim), got_ext = (n, 4)
    uint32 [geometry, instance, custom, hit kind] or None."""
    gi = None if got_ext is None else got_ext[:, 1]
    gg = None if got_ext is None else got_ext[:, 0]
    cls = classify_hits(S, rays, got["prim"], got["t"], got["u"], got["v"], exp, got_instance=gi, got_geometry=gg,
                        exact=exact, **kw)
    return cls, counts(cls)


def classify_wavefront(S, cam, width, height, light, got, exp, sample_index=0, tlas=0, watertight=False,
                       threads=16, row0=0) -> dict:
    """Pixel records of the primary + shadow + bounce workload (rdn_pixel_result)
    of rows [row0, row0 + len(got) / width) against the oracle's records `exp`
    of the same rows, both with the same triangle test. Per ray class:
      primary  identical / tie / nan / edge / other
      shadow   (pixels whose primary is identical) hit/miss: identical / nan / other,
               plus `direct` (the shading value) bit-identical where visible
      bounce   (pixels whose primary is identical) identical / tie / nan / edge / other
      secondary_after_primary_difference: pixels whose primary differs (a tie or
               a NaN exposure), so that their shadow and bounce rays are other rays."""
    n = len(got)
    pix = np.arange(n, dtype=np.uint32) + np.uint32(row0 * width)
    bits = lambda a: np.ascontiguousarray(a, np.float32).view(np.uint32)  # noqa: E731
    # cheap prefilter: only pixels with any difference need the rays
    diff = ((got["primary_prim"] != exp["primary_prim"]) | (bits(got["primary_t"]) != bits(exp["primary_t"]))
            | (got["light"] != exp["light"]) | (bits(got["direct"]) != bits(exp["direct"]))
            | (got["bounce_prim"] != exp["bounce_prim"]) | (bits(got["bounce_t"]) != bits(exp["bounce_t"])))
    idx = np.nonzero(diff)[0]
    res = {"pixels": n, "primary": counts(np.zeros(n, np.int8))}
    prim_cls = np.zeros(n, np.int8)
    sh_cls = np.zeros(n, np.int8)
    bo_cls = np.zeros(n, np.int8)
    direct_mismatch = 0
    if idx.size:
        r_p, r_s, r_b, has = orc.wavefront_pixel_rays(S, cam.as_floats(), width, height, light, pix[idx],
                                                      sample_index, tlas, threads=threads, watertight=watertight)
        g, e = got[idx], exp[idx]
        # primary: instance from the record, geometry 0 (one geometry per BLAS in these scenes)
        eh = np.zeros(idx.size, orc.HIT_DTYPE)
        eh["prim"], eh["t"], eh["instance"] = e["primary_prim"], e["primary_t"], e["primary_instance"]
        eh["u"] = eh["v"] = 0.0
        c = classify_hits(S, r_p, g["primary_prim"], g["primary_t"], np.zeros(idx.size, np.float32),
                          np.zeros(idx.size, np.float32), eh, got_instance=g["primary_instance"],
                          got_geometry=np.zeros(idx.size, np.uint32), tlas_uniform=tlas, threads=threads)
        prim_cls[idx] = c
        ok = c == IDENTICAL
        # shadow: hit/miss (light 1 visible, 2 occluded) where the primary is identical
        sel = np.nonzero(ok & has)[0]
        if sel.size:
            sh = np.zeros(sel.size, orc.HIT_DTYPE)
            sh["prim"] = np.where(e["light"][sel] == 2, 0, orc.MISS)
            cs = classify_hits(S, r_s[sel], np.where(g["light"][sel] == 2, 0, orc.MISS).astype(np.uint32),
                               np.zeros(sel.size, np.float32), np.zeros(sel.size, np.float32),
                               np.zeros(sel.size, np.float32), sh, first_hit=True, tlas_uniform=tlas,
                               ray_flags=0x04, threads=threads)
            sh_cls[idx[sel]] = cs
            vis = (cs == IDENTICAL) & (e["light"][sel] == 1)
            direct_mismatch = int((bits(g["direct"][sel][vis]) != bits(e["direct"][sel][vis])).sum())
            bh = np.zeros(sel.size, orc.HIT_DTYPE)
            bh["prim"], bh["t"] = e["bounce_prim"][sel], e["bounce_t"][sel]
            bh["instance"] = 0
            cb = classify_hits(S, r_b[sel], g["bounce_prim"][sel], g["bounce_t"][sel], np.zeros(sel.size, np.float32),
                               np.zeros(sel.size, np.float32), bh, got_instance=np.zeros(sel.size, np.uint32),
                               got_geometry=np.zeros(sel.size, np.uint32), tlas_uniform=tlas, threads=threads)
            bo_cls[idx[sel]] = cb
    prim_ok = prim_cls == IDENTICAL
    has_sec = prim_ok & (exp["primary_prim"] != orc.MISS)
    res["primary"] = counts(prim_cls)
    sc = counts(sh_cls[has_sec])
    res["shadow"] = {k: sc[k] for k in ("n", "identical", "nan", "other")}
    res["bounce"] = counts(bo_cls[has_sec])
    res["direct_mismatch"] = direct_mismatch
    res["secondary_after_primary_difference"] = int(((~prim_ok) & (exp["primary_prim"] != orc.MISS)).sum())
    res["other"] = res["primary"]["other"] + res["shadow"]["other"] + res["bounce"]["other"] + direct_mismatch
    return res
