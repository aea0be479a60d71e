"""The path-tracing oracle (oracle/orc_pt.h) on the CPU: its fixed-polynomial
functions against float64 numpy, the physical surface against the reference's
construction rules (direct_lighting.rs:14-59, surface_bridge.rs:171-224), the
bsdf / pdf / importance sample against a float64 restatement of the reference
formulas (microfacet/device/{mod,diffuse,specular}.rs), the tone maps
(tonemap.rs) and a one-bounce frame whose pixel radiance is recomputed here
from the same seeds (ray_hit.rs:12-103, ray_gen.rs:101-150)."""

import numpy as np
import pytest

from helpers import orc, single_mesh_scene
from rendiation_gb300 import path_tracing as pt
from rendiation_gb300 import scenes
from rendiation_gb300 import task_graph as tg


def test_polynomial_functions_against_float64():
    x = np.concatenate([np.linspace(0, 3, 3001), np.geomspace(1e-6, 1e7, 2000)]).astype(np.float32)
    assert np.max(np.abs(orc.pt_math("atan", x) - np.arctan(x.astype(np.float64)))) < 3e-7
    y = np.geomspace(1e-30, 1e30, 4001).astype(np.float32)
    assert np.max(np.abs(orc.pt_math("log2", y) - np.log2(y.astype(np.float64)))) < 4e-6
    e = np.linspace(-125, 127, 5001).astype(np.float32)
    assert np.max(np.abs(orc.pt_math("exp2", e) / np.exp2(e.astype(np.float64)) - 1)) < 1e-6
    p = np.geomspace(1e-8, 1e6, 4001).astype(np.float32)
    # f32 exp2(2.2 log2 x): the log carries ~1e-7 of |log2 x|, so the error grows with |log2 x|
    assert np.max(np.abs(orc.pt_math("pow22", p) / p.astype(np.float64) ** 2.2 - 1)) < 5e-6
    assert orc.pt_math("pow22", np.zeros(1))[0] == 0.0
    assert np.isinf(orc.pt_math("exp2", np.array([200.0]))[0]) and orc.pt_math("exp2", np.array([-200.0]))[0] == 0


def surface64(m):
    """PhysicalShading + surface point, float64 (direct_lighting.rs:14-59, surface_bridge.rs:171-224)."""
    base = np.asarray(m["base_color"], np.float64)
    if int(m["workflow"]) == 1:
        spec = np.asarray(m["specular"], np.float64)
        albedo, f0 = base * (1 - spec.max()), spec
    else:
        met, refl = float(m["metallic"]), float(m["reflectance"])
        f0 = base * met + 0.16 * refl * refl * (1 - met)
        albedo = base * (1 - met)
    alpha = float(m["perceptual_roughness"]) ** 2
    est = 0.2 * (1 - f0.max()) + f0.max()
    return albedo, f0, alpha, est


def ggx_d64(alpha, n, h):
    noh = max(n @ h, 1e-4)
    r2 = alpha * alpha
    d = (noh * r2 - noh) * noh + 1
    return r2 / (np.pi * d * d)


def bsdf64(surf, v, l, n):
    albedo, f0, alpha, est = surf
    h = (l + v) / np.linalg.norm(l + v)
    f = f0 + (1 - f0) * (1 - v @ h) ** 5
    nl, nv = max(l @ n, 1e-4), max(v @ n, 1e-4)
    r2 = alpha * alpha
    g = 0.5 / (nv * np.sqrt(nv * (nv - nv * r2) + r2) + nl * np.sqrt(nl * (nl - nl * r2) + r2)) * 4 * nl * nv
    spec = ggx_d64(alpha, n, h) * g * f / (4 * nl * nv)
    return albedo / np.pi * (1 - est) + spec * est


def pdf64(surf, v, l, n):
    _, _, alpha, est = surf
    m = (v + l) / np.linalg.norm(v + l)
    spec = (n @ m) * ggx_d64(alpha, n, m) / (4 * abs(m @ v))
    return max(l @ n, 0) / np.pi * (1 - est) + spec * est


def materials():
    return np.array([pt.metallic_material((0.8, 0.6, 0.3), 0.7, 0.0, 0.5),
                     pt.metallic_material((0.9, 0.9, 0.95), 0.25, 1.0),
                     pt.specular_material((0.2, 0.5, 0.7), 0.4, (0.3, 0.2, 0.1)),
                     pt.metallic_material((0.5, 0.5, 0.5), 0.9, 0.3, 0.2)], pt.MATERIAL_DTYPE)


def test_surface_construction():
    mats = materials()
    for k, m in enumerate(mats):
        _, _, (albedo, f0, alpha, est) = orc.pt_surface_query(1, [0, 0, 1], [0, 0, 1], [0, 0, 1], mats,
                                                               sm_id=k)
        a64, f64, al64, e64 = surface64(m)
        assert np.allclose(albedo, a64, rtol=1e-6) and np.allclose(f0, f64, rtol=1e-6)
        assert alpha == pytest.approx(al64, rel=1e-6) and est == pytest.approx(e64, rel=1e-6)
    # default material (no table, or an index outside it): base 0.5, roughness 0.5, metallic 0, reflectance 0.5
    for kw in ({}, {"materials": mats, "sm_id": 99}, {"materials": mats, "sm_to_material": [3, 7], "sm_id": 1},
               {"materials": mats, "sm_to_material": [3], "sm_id": 1}):
        _, _, (albedo, f0, alpha, est) = orc.pt_surface_query(1, [0, 0, 1], [0, 0, 1], [0, 0, 1], **kw)
        assert np.allclose(albedo, 0.5) and np.allclose(f0, 0.04) and alpha == 0.25
        assert est == pytest.approx(0.2 * 0.96 + 0.04, rel=1e-6)
    # the table routes custom index 0 to material 3
    _, _, s3 = orc.pt_surface_query(1, [0, 0, 1], [0, 0, 1], [0, 0, 1], mats, sm_to_material=[3], sm_id=0)
    assert np.allclose(s3[1], surface64(mats[3])[1], rtol=1e-6)


def test_bsdf_and_pdf_against_float64():
    rng = np.random.default_rng(4)
    mats = materials()
    for k in range(400):
        m = mats[k % len(mats)]
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        v = rng.normal(size=3)
        v = v if v @ n > 0 else -v
        v /= np.linalg.norm(v)
        l2 = rng.normal(size=3)
        l2 = l2 if l2 @ n > 0.05 else -l2
        l2 /= np.linalg.norm(l2)
        if l2 @ n < 0.05 or v @ n < 0.05:
            continue
        _, (b2, p2), _ = orc.pt_surface_query(k, v, n, l2, mats, sm_id=k % len(mats))
        surf = surface64(m)
        assert np.allclose(b2, bsdf64(surf, v, l2, n), rtol=2e-4, atol=1e-7), k
        assert p2 == pytest.approx(pdf64(surf, v, l2, n), rel=2e-4, abs=1e-7), k


def pcg_states(seed):
    state = seed

    def nxt():
        nonlocal state
        prev = (state * 747796405 + 2891336453) & 0xFFFFFFFF
        word = (((prev >> ((prev >> 28) + 4)) ^ prev) * 277803737) & 0xFFFFFFFF
        state = prev
        r = ((word >> 22) ^ word) & 0xFFFFFFFF
        return float(np.array(0x3F800000 | (r >> 9), np.uint32).view(np.float32)) - 1.0

    return nxt


def xxhash32(x, y, z):
    p0, p1, p2, p3 = 2246822519, 3266489917, 668265263, 374761393
    m = 0xFFFFFFFF
    h = (z + p3 + x * p1) & m
    h = (p2 * (((h << 17) | (h >> 15)) & m)) & m
    h = (h + y * p1) & m
    h = (p2 * (((h << 17) | (h >> 15)) & m)) & m
    h = (p0 * (h ^ (h >> 15))) & m
    h = (p1 * (h ^ (h >> 13))) & m
    return h ^ (h >> 16)


def concentric64(sx, sy):
    ux, uy = 2 * sx - 1, 2 * sy - 1
    if ux == 0 and uy == 0:
        return 0.0, 0.0
    if abs(ux) > abs(uy):
        r, th = ux, np.pi / 4 * (uy / ux)
    else:
        r, th = uy, np.pi / 2 - np.pi / 4 * (ux / uy)
    return np.cos(th) * r, np.sin(th) * r


def tbn64(n):
    sign = -1.0 if n[2] < 0 else 1.0
    a = -1 / (sign + n[2])
    b = n[0] * n[1] * a
    t = np.array([1 + sign * n[0] * n[0] * a, sign * b, -sign * n[0]])
    bt = np.array([b, sign + n[1] * n[1] * a, -n[1]])
    return np.stack([t / np.linalg.norm(t), bt / np.linalg.norm(bt), n], 1)


def sample64(surf, v, n, seed):
    nxt = pcg_states(seed)
    _, _, alpha, est = surf
    if nxt() < est:
        u = nxt()
        th = np.arctan(alpha * np.sqrt(u / (1 - u)))
        x, y = concentric64(nxt(), nxt())
        m = tbn64(n) @ np.array([x * np.sin(th), y * np.sin(th), np.cos(th)])
        i = -v
        return i - 2 * (m @ i) * m
    x, y = concentric64(nxt(), nxt())
    return tbn64(n) @ np.array([x, y, np.sqrt(1 - x * x - y * y)])


def test_importance_sample_against_float64():
    rng = np.random.default_rng(5)
    mats = materials()
    spec_seen = diff_seen = 0
    for k in range(600):
        m = mats[k % len(mats)]
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        v = rng.normal(size=3)
        v = v if v @ n > 0.1 else -v
        v /= np.linalg.norm(v)
        seed = int(rng.integers(0, 2**32))
        (l, b, p), (b2, p2), _ = orc.pt_surface_query(seed, v, n, [0, 0, 1], mats, sm_id=k % len(mats))
        surf = surface64(m)
        l64 = sample64(surf, v, n, seed)
        if not np.all(np.isfinite(l64)) or abs(l64 @ n) < 1e-3:
            continue
        assert np.allclose(l, l64, atol=2e-5), (k, l, l64)
        spec_seen += pcg_states(seed)() < surf[3]
        diff_seen += pcg_states(seed)() >= surf[3]
        # the bsdf and pdf of the sample are those of its direction
        (_, (b3, p3), _) = orc.pt_surface_query(seed, v, n, l, mats, sm_id=k % len(mats))
        assert np.array_equal(b, b3) and p == p3
    assert spec_seen > 100 and diff_seen > 100


@pytest.mark.parametrize("tone", [pt.TONE_MAP_NONE, pt.TONE_MAP_LINEAR, pt.TONE_MAP_REINHARD, pt.TONE_MAP_CINEON,
                                  pt.TONE_MAP_ACES_FILMIC])
def test_tone_maps_against_float64(tone):
    x = np.concatenate([[0.0], np.geomspace(1e-4, 50, 400)]).astype(np.float32)
    got = orc.pt_math("tone", x, arg=tone)
    c = x.astype(np.float64)
    if tone in (pt.TONE_MAP_NONE, pt.TONE_MAP_LINEAR):
        want = c
    elif tone == pt.TONE_MAP_REINHARD:
        want = np.clip(c / (1 + c), 0, 1)
    elif tone == pt.TONE_MAP_CINEON:
        e = np.maximum(c - 0.004, 0)
        want = ((e * (6.2 * e + 0.5)) / (e * (6.2 * e + 1.7) + 0.06)) ** 2.2
    else:
        mi = np.array([[0.59719, 0.35458, 0.04823], [0.07600, 0.90834, 0.01566], [0.02840, 0.13383, 0.83777]])
        mo = np.array([[1.60475, -0.53108, -0.07367], [-0.10208, 1.10813, -0.00605], [-0.00327, -0.07276, 1.07602]])
        v = (mi @ np.stack([c, c, c]) / 0.6)
        v = (v * (v + 0.0245786) - 0.000090537) / (v * (0.983729 * v + 0.432951) + 0.238081)
        want = np.clip((mo @ v)[0], 0, 1)
    assert np.allclose(got, want, rtol=3e-5, atol=3e-6)


def test_clamp_size_by_area():
    assert pt.clamp_size_by_area(1920, 1080) == (682, 384)
    assert pt.clamp_size_by_area(512, 512) == (512, 512)
    assert pt.clamp_size_by_area(100, 50) == (724, 362)
    assert pt.clamp_size_by_area(1, 1, 1) == (1, 1)


def test_one_bounce_frame_against_float64():
    """max_path_depth 1 over a flat floor lit by one directional light, black
    background: each pixel's radiance is throughput * sampled radiance of its
    first hit, recomputed here in float64 from the pixel's two seeds."""
    W, H = 24, 16
    g = 8
    xs = np.linspace(-2, 2, g + 1)
    pos = np.array([[x, y, 0.0] for y in xs for x in xs], np.float32)
    idx = []
    for j in range(g):
        for i in range(g):
            a = j * (g + 1) + i
            idx += [a, a + 1, a + g + 2, a, a + g + 2, a + g + 1]
    mesh = scenes.Mesh(pos, np.array(idx, np.uint32))
    S = single_mesh_scene(mesh).build_oracle()
    eye = np.array([0.1, -0.8, 1.2], np.float32)
    vp = tg.look_at_view_projection_inv(eye, (0.0, 0.0, 0.0), (0, 0, 1), 50.0, W / H)
    mats = materials()[:1]
    light = pt.directional_light((2.0, 1.5, 1.0), (0.3, 0.2, -1.0))
    img = np.zeros(W * H, np.uint32)
    rad = np.zeros(W * H * 4, np.float32)
    rays, _ = orc.pt_render(S, vp, eye, W, H, img, lights=[light], materials=mats, max_depth=1,
                            tone_map=pt.TONE_MAP_NONE, sample_count=5, radiance=rad, threads=4)
    rad = rad.reshape(H, W, 4)
    assert rays == (W * H, W * H)  # every camera ray hits the floor; one shadow ray each, none occluded
    surf = surface64(mats[0])
    ldir = -np.asarray(light["direction"], np.float64)
    E = np.asarray(light["illuminance"], np.float64)
    for y in range(H):
        for x in range(W):
            # the floor's shading normal faces the camera: +z
            n = np.array([0.0, 0.0, 1.0])
            # camera ray (ray_gen.rs / camera.rs) in float64 for the view direction
            nx = pcg_states(xxhash32(x, y, 5))
            ux, uy = x / W + nx() / W, y / H + nx() / H
            r = np.asarray(vp, np.float64).reshape(4, 4).T @ np.array([2 * ux - 1, -(2 * uy - 1), 1.0, 1.0])
            d = r[:3] / r[3] - eye
            d /= np.linalg.norm(d)
            v = -d
            l = sample64(surf, v, n, xxhash32(x, y, 15))
            thr = (l @ n) * bsdf64(surf, v, l, n) / max(pdf64(surf, v, l, n), 1e-4)
            sampled = abs(n @ ldir) * bsdf64(surf, v, ldir, n) * E
            want = thr * sampled
            assert np.allclose(rad[y, x, :3], want, rtol=2e-3, atol=1e-6), (x, y, rad[y, x], want)
            assert rad[y, x, 3] == 1.0
    # the RGBA8 texel is the first sample's value (old texel 0, count 5: (0 * 5 + ldr) / 6)
    q = np.clip(rad[..., :3].reshape(-1, 3) / 6.0, 0, 1) * 255
    got = np.stack([img & 0xFF, (img >> 8) & 0xFF, (img >> 16) & 0xFF], 1)
    assert np.max(np.abs(got - np.rint(q))) <= 1
    assert np.all((img >> 24) == 255)


def env_sample64(cube, m, d, intensity):
    """Cube-map lookup in float64: M (d, 1) / w, the major axis's face, bilinear over texel centres clamped to
    the face (the convention rdn_pt_desc.env_cube documents)."""
    r = m @ np.array([d[0], d[1], d[2], 1.0])
    x, y, z = r[:3] / r[3]
    ax, ay, az = abs(x), abs(y), abs(z)
    if ax >= ay and ax >= az:
        face, sc, tc, ma = (0, -z, -y, ax) if x >= 0 else (1, z, -y, ax)
    elif ay >= az:
        face, sc, tc, ma = (2, x, z, ay) if y >= 0 else (3, x, -z, ay)
    else:
        face, sc, tc, ma = (4, x, -y, az) if z >= 0 else (5, -x, -y, az)
    n = cube.shape[1]
    u = (sc / ma + 1) / 2 * n - 0.5
    v = (tc / ma + 1) / 2 * n - 0.5
    i0, j0 = int(np.floor(u)), int(np.floor(v))
    fu, fv = u - i0, v - j0
    c = lambda i, j: cube[face, min(max(j, 0), n - 1), min(max(i, 0), n - 1), :3].astype(np.float64)
    top = c(i0, j0) * (1 - fu) + c(i0 + 1, j0) * fu
    bot = c(i0, j0 + 1) * (1 - fu) + c(i0 + 1, j0 + 1) * fu
    return (top * (1 - fv) + bot * fv) * intensity


def test_env_cube_background_against_float64():
    """Camera rays that all miss sample the environment cube (PTRayMissCtx::EnvCube): each pixel's radiance
    against a float64 lookup of the same direction."""
    W, H = 24, 18
    mesh = scenes.Mesh(np.array([[50, 50, 50], [51, 50, 50], [50, 51, 50]], np.float32), np.arange(3, dtype=np.uint32))
    S = single_mesh_scene(mesh).build_oracle()
    rng = np.random.default_rng(9)
    cube = rng.random((6, 8, 8, 4)).astype(np.float32)
    a = 0.6
    rot = np.array([[np.cos(a), -np.sin(a), 0, 0], [np.sin(a), np.cos(a), 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
    for eye, target in (((0, 0, 0), (1, 0.2, 0.1)), ((0, 0, 0), (-0.3, -1, 0.4)), ((0, 0, 0), (0.2, 0.1, -1))):
        vp = tg.look_at_view_projection_inv(eye, target, (0, 0, 1) if abs(target[2]) < 0.9 else (0, 1, 0), 100.0,
                                            W / H)
        img = np.zeros(W * H, np.uint32)
        rad = np.zeros(W * H * 4, np.float32)
        orc.pt_render(S, vp, np.asarray(eye, np.float32), W, H, img, max_depth=3, tone_map=pt.TONE_MAP_NONE,
                      background=pt.BACKGROUND_ENV_CUBE, env_cube=cube, env_transform=rot, env_intensity=1.5,
                      radiance=rad, threads=2)
        rad = rad.reshape(H, W, 4)
        assert np.all(rad[..., 3] == 1.0)  # one core ray each, a miss
        for y in range(H):
            for x in range(W):
                nx = pcg_states(xxhash32(x, y, 0))
                ux, uy = x / W + nx() / W, y / H + nx() / H
                r = np.asarray(vp, np.float64).reshape(4, 4).T @ np.array([2 * ux - 1, -(2 * uy - 1), 1.0, 1.0])
                d = r[:3] / r[3] - np.asarray(eye, np.float64)
                d /= np.linalg.norm(d)
                want = env_sample64(cube, rot, d, 1.5)
                assert np.allclose(rad[y, x, :3], want, atol=2e-4), (x, y, rad[y, x], want)


def test_env_cube_faces_and_texel_centres():
    """Directions through texel centres of each face return the texel itself (times the intensity)."""
    mesh = scenes.Mesh(np.array([[50, 50, 50], [51, 50, 50], [50, 51, 50]], np.float32), np.arange(3, dtype=np.uint32))
    S = single_mesh_scene(mesh).build_oracle()
    cube = np.zeros((6, 2, 2, 4), np.float32)
    for f in range(6):
        cube[f, :, :, :3] = (f + 1) / 10.0
    # a 1x1 frame looking straight along each axis: the ray passes the face centre (4 texels of equal value)
    for f, (target, up) in enumerate((((1, 0, 0), (0, 0, 1)), ((-1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1)),
                                      ((0, -1, 0), (0, 0, 1)), ((0, 0, 1), (0, 1, 0)), ((0, 0, -1), (0, 1, 0)))):
        vp = tg.look_at_view_projection_inv((0, 0, 0), target, up, 1.0, 1.0)
        img = np.zeros(1, np.uint32)
        rad = np.zeros(4, np.float32)
        orc.pt_render(S, vp, np.zeros(3, np.float32), 1, 1, img, tone_map=pt.TONE_MAP_NONE,
                      background=pt.BACKGROUND_ENV_CUBE, env_cube=cube, env_intensity=2.0, radiance=rad, threads=1)
        assert np.allclose(rad[:3], 2.0 * (f + 1) / 10.0, rtol=1e-6), (f, rad)
