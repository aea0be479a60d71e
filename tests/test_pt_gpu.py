"""The reference path tracer (feature/path_tracing: ray_gen.rs, ray_hit.rs,
ray_miss.rs, the lighting and surface bridges) as the fused CUDA frame
(rdn_path_tracing_render) against the path-tracing oracle (oracle/orc_pt.h),
over progressive samples. The reference traversal order: every RGBA8 texel and
every HDR radiance bit-identical (NaN equal to NaN); the four-child walk:
identical except pixels whose path meets an exact-distance tie."""

import ctypes

import numpy as np
import pytest

import naive_fixture as nf
from helpers import instanced_scene, orc, single_mesh_scene
from rendiation_gb300 import native
from rendiation_gb300 import path_tracing as pt
from rendiation_gb300 import raytracing as rt
from rendiation_gb300 import scenes
from rendiation_gb300 import task_graph as tg

pytestmark = pytest.mark.gpu

W, H = 77, 45  # not a multiple of the 4x8 tile: the last tiles overhang the frame
SAMPLES = (0, 1, 2)


def vertex_normals(mesh):
    p = mesh.positions.astype(np.float64)
    t = mesh.indices.reshape(-1, 3)
    fn = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, t[:, k], fn)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return n.astype(np.float32)


MATERIALS = np.array([pt.metallic_material((0.8, 0.6, 0.3), 0.7, 0.0, 0.5),
                      pt.metallic_material((0.9, 0.9, 0.95), 0.25, 1.0),
                      pt.specular_material((0.2, 0.5, 0.7), 0.4, (0.3, 0.2, 0.1)),
                      pt.metallic_material((0.5, 0.5, 0.5), 0.05, 0.3, 0.2)], pt.MATERIAL_DTYPE)
LIGHTS = np.array([pt.directional_light((3.0, 2.5, 2.0), (0.3, 0.2, -1.0)),
                   pt.directional_light((0.5, 0.7, 1.2), (-0.6, 0.4, -0.5)),
                   pt.directional_light((1.0, 1.0, 1.0), (0.0, -0.2, -1.0))], pt.DIRECTIONAL_LIGHT_DTYPE)


def field():
    mesh = scenes.heightfield(48, seed=3, jitter_sigma=0.02)
    eye = (0.5, -0.45, 0.75)
    vp = tg.look_at_view_projection_inv(eye, (0.5, 0.5, 0.0), (0, 0, 1), 45.0, W / H)
    return single_mesh_scene(mesh), mesh, vp, np.asarray(eye, np.float32)


def instanced():
    eye = (0.4, -2.6, 1.6)
    vp = tg.look_at_view_projection_inv(eye, (0.4, 0.4, 0.3), (0, 0, 1), 50.0, W / H)
    return instanced_scene(seed=2), None, vp, np.asarray(eye, np.float32)


def fixture():
    eye = (0.0, 0.0, 0.0)
    vp = tg.look_at_view_projection_inv(eye, (0.0, 0.0, -1.0), (0, 1, 0), 90.0, W / H)
    return nf.make_scene(), None, vp, np.asarray(eye, np.float32)


SCENES = {"field": field, "instanced": instanced, "fixture": fixture}


def run_pair(scene_fn, traversal=rt.TRAVERSAL_REFERENCE, with_normals=False, samples=SAMPLES, tlas=0, **kw):
    import torch

    scene, mesh, vp, eye = scene_fn()
    normals = vertex_normals(mesh) if with_normals else None
    S = scene.build_oracle()
    img = np.zeros(W * H, np.uint32)
    rad = np.zeros(W * H * 4, np.float32)
    rays = [0, 0]
    okw = {k: v for k, v in kw.items() if k not in ("block_size", "schedule", "register_tier", "speculation")}
    for s in samples:
        r, _ = orc.pt_render(S, vp, eye, W, H, img, sample_count=s, normals=normals, radiance=rad, tlas=tlas,
                             intersector=1 if traversal & rt.INTERSECT_WATERTIGHT else 0, threads=8, **okw)
        rays[0] += r[0]
        rays[1] += r[1]
    P = scene.build_product()
    nt = None if normals is None else torch.from_numpy(normals.reshape(-1)).cuda()
    rk = dict(kw)
    renames = {"max_depth": "max_path_depth", "bg": "background_color"}
    rk = {renames.get(k, k): v for k, v in rk.items()}
    R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, normals=nt, traversal=traversal, tlas_uniform=tlas,
                                              keep_radiance=True, count_rays=True, **rk)
    for s in samples:
        R.sample_count = s
        R.render()
    torch.cuda.synchronize()
    assert P.check_errors() == (0, 0)
    got = R.result().reshape(-1, 4).astype(np.uint32)
    packed = got[:, 0] | (got[:, 1] << 8) | (got[:, 2] << 16) | (got[:, 3] << 24)
    grad = R.radiance.cpu().numpy()
    return img, rad, packed, grad, tuple(rays), R.rays_traced()


def same_bits(a, b):
    a, b = a.copy(), b.copy()
    nan = np.isnan(a) & np.isnan(b)
    a[nan] = 0
    b[nan] = 0
    return a.view(np.uint32) == b.view(np.uint32)


# The reference's fixture runs with the watertight test: its sphere's zero-area
# pole triangles give NaN distances under the reference's formula, and a NaN
# hit position's bits (which differ between host and device NaNs) feed
# offset_ray_hit's integer offset.
@pytest.mark.parametrize("name,normals,tone", [
    ("field", True, pt.TONE_MAP_ACES_FILMIC),
    ("field", False, pt.TONE_MAP_REINHARD),
    ("instanced", False, pt.TONE_MAP_ACES_FILMIC),
    ("instanced", False, pt.TONE_MAP_CINEON),
    ("fixture", False, pt.TONE_MAP_LINEAR),
    ("fixture", False, pt.TONE_MAP_NONE),
])
def test_reference_order_is_bit_identical(cuda, name, normals, tone):
    sm = [0, 1, 2, 3, 0, 1, 2, 3, 9, 1, 2, 3] if name == "instanced" else None
    fixture_kw = dict(tlas=4, traversal=rt.TRAVERSAL_REFERENCE | rt.INTERSECT_WATERTIGHT) if name == "fixture" else {}
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        SCENES[name], with_normals=normals, tone_map=tone, lights=LIGHTS, materials=MATERIALS, sm_to_material=sm,
        bg=(0.05, 0.1, 0.2), exposure=1.3, **fixture_kw)
    assert np.array_equal(img, want_img)
    assert same_bits(rad, want_rad).all()
    assert rays_g == rays_o
    r = want_rad.reshape(-1, 4)
    # paths of every length up to 3, lit and shadowed pixels, some escaped to the background
    assert set(np.unique(r[:, 3]).astype(int)) >= {1, 2, 3}
    assert rays_o[1] > 0 and len(np.unique(want_img)) > 50


def test_test_background_without_lights(cuda):
    """PTRayMissCtx::Test and no light: no shadow ray, every pixel's radiance is
    the throughput of its escaping path times 0.7 or 0.3."""
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        field, lights=None, materials=MATERIALS, background=pt.BACKGROUND_TEST, tone_map=pt.TONE_MAP_LINEAR)
    assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()
    assert rays_o[1] == 0 and rays_g == rays_o


@pytest.mark.parametrize("depth", [0, 1, 5])
def test_path_depth(cuda, depth):
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        instanced, max_depth=depth, lights=LIGHTS[:1], materials=MATERIALS, bg=(0.3, 0.3, 0.3))
    assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()
    assert rays_g == rays_o
    assert np.max(want_rad.reshape(-1, 4)[:, 3]) == depth


def test_watertight_intersector(cuda):
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        field, traversal=rt.TRAVERSAL_REFERENCE | rt.INTERSECT_WATERTIGHT, with_normals=True, lights=LIGHTS,
        materials=MATERIALS)
    assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE])
def test_ordered_walks_match_except_ties(cuda, traversal):
    want_img, want_rad, img, rad, _, _ = run_pair(instanced, traversal=traversal, lights=LIGHTS, materials=MATERIALS)
    assert (img == want_img).mean() > 0.995
    assert same_bits(rad, want_rad).reshape(-1, 4).all(1).mean() > 0.995


@pytest.mark.parametrize("speculation", [4, 16])
def test_leaf_postponement_threshold(cuda, speculation):
    want_img, want_rad, img, rad, _, _ = run_pair(instanced, traversal=rt.TRAVERSAL_ORDERED_WIDE, lights=LIGHTS,
                                                  materials=MATERIALS, speculation=speculation)
    assert (img == want_img).mean() > 0.995
    assert same_bits(rad, want_rad).reshape(-1, 4).all(1).mean() > 0.995


@pytest.mark.parametrize("name", ["field", "instanced"])
def test_schedules_change_no_pixel(cuda, name):
    """One thread per pixel, persistent warps refilled with pixels as paths
    end, and wavefront passes over path queues compute every pixel with the
    same operations, at every register budget."""
    a = run_pair(SCENES[name], traversal=rt.TRAVERSAL_ORDERED_WIDE, lights=LIGHTS, materials=MATERIALS,
                 schedule=pt.SCHEDULE_PIXEL)
    for sched in (pt.SCHEDULE_REFILL, pt.SCHEDULE_WAVEFRONT):
        for tier in (0, 1, 2):
            c = run_pair(SCENES[name], traversal=rt.TRAVERSAL_ORDERED_WIDE, lights=LIGHTS, materials=MATERIALS,
                         schedule=sched, register_tier=tier)
            assert np.array_equal(a[2], c[2]) and same_bits(a[3], c[3]).all() and a[5] == c[5], (sched, tier)


@pytest.mark.parametrize("lights", [None, LIGHTS[:1]])
@pytest.mark.parametrize("depth", [0, 1, 5])
def test_wavefront_schedule_matches_the_oracle(cuda, lights, depth):
    """The wavefront passes in the reference order: without lights every pass
    traces core rays, with lights the passes alternate core and shadow rays."""
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        instanced, max_depth=depth, lights=lights, materials=MATERIALS, bg=(0.3, 0.3, 0.3),
        schedule=pt.SCHEDULE_WAVEFRONT)
    assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()
    assert rays_g == rays_o


@pytest.mark.parametrize("block_size", [32, 64])
def test_block_size_changes_no_pixel(cuda, block_size):
    a = run_pair(field, traversal=rt.TRAVERSAL_ORDERED_WIDE, lights=LIGHTS, materials=MATERIALS)
    b = run_pair(field, traversal=rt.TRAVERSAL_ORDERED_WIDE, lights=LIGHTS, materials=MATERIALS,
                 block_size=block_size)
    assert np.array_equal(a[2], b[2]) and same_bits(a[3], b[3]).all()


def test_invalid_descriptors_are_rejected(cuda):
    import torch

    scene, _, vp, eye = field()
    P = scene.build_product()
    bad = [dict(tone_map=5), dict(background=2), dict(max_path_depth=65), dict(schedule=3), dict(register_tier=3)]
    for kw in bad:
        R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, **kw)
        with pytest.raises(native.RdnError):
            R.render()
    R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, keep_radiance=True)
    d = R.desc()
    d.radiance = R.radiance.data_ptr() + 4  # not 16-byte aligned
    assert P._L.rdn_path_tracing_render(P._h, ctypes.byref(d), None) == -1  # RDN_ERR_INVALID_ARG
    d = R.desc()
    d.light_count = 2  # with a null light array
    assert P._L.rdn_path_tracing_render(P._h, ctypes.byref(d), None) == -1  # RDN_ERR_INVALID_ARG
    d = R.desc()
    d.image = None
    assert P._L.rdn_path_tracing_render(P._h, ctypes.byref(d), None) == -1  # RDN_ERR_INVALID_ARG
    R.schedule = pt.SCHEDULE_WAVEFRONT
    d = R.desc()
    d.scratch_bytes -= 256  # too small
    assert P._L.rdn_path_tracing_render(P._h, ctypes.byref(d), None) == -1  # RDN_ERR_INVALID_ARG
    d = R.desc()
    d.scratch += 16  # not 256-byte aligned
    assert P._L.rdn_path_tracing_render(P._h, ctypes.byref(d), None) == -1  # RDN_ERR_INVALID_ARG
    torch.cuda.synchronize()
    assert int(R.image.sum().item()) == 0  # nothing was written


def test_render_accumulates_and_resets(cuda):
    import torch

    scene, _, vp, eye = field()
    P = scene.build_product()
    R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, lights=LIGHTS, materials=MATERIALS,
                                              traversal=rt.TRAVERSAL_ORDERED_WIDE)
    for _ in range(4):
        R.render()
    torch.cuda.synchronize()
    assert R.sample_count == 4
    first = R.result().copy()
    R.reset_sample()
    for _ in range(4):
        R.render()
    torch.cuda.synchronize()
    assert np.array_equal(R.result(), first)
    assert np.all(first[..., 3] == 255)


@pytest.mark.parametrize("schedule", [pt.SCHEDULE_PIXEL, pt.SCHEDULE_REFILL, pt.SCHEDULE_WAVEFRONT])
def test_environment_cube_background(cuda, schedule):
    """PTRayMissCtx::EnvCube: escaping paths sample a rotated, scaled cube map;
    every texel and radiance bit-identical to the oracle in reference order."""
    rng = np.random.default_rng(12)
    cube = rng.random((6, 16, 16, 4)).astype(np.float32)
    a = 0.9
    rot = np.array([[1, 0, 0, 0], [0, np.cos(a), -np.sin(a), 0], [0, np.sin(a), np.cos(a), 0], [0, 0, 0, 1]])
    want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
        field, with_normals=True, lights=LIGHTS[:2], materials=MATERIALS, background=pt.BACKGROUND_ENV_CUBE,
        env_cube=cube, env_transform=rot, env_intensity=1.7, schedule=schedule)
    assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()
    assert rays_g == rays_o
    # some paths escaped to the environment
    assert len(np.unique(want_rad.reshape(-1, 4)[:, 3])) > 1


def test_environment_cube_needs_a_map(cuda):
    scene, _, vp, eye = field()
    P = scene.build_product()
    R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, background=pt.BACKGROUND_ENV_CUBE)
    with pytest.raises(native.RdnError):
        R.render()


@pytest.mark.parametrize("schedule", [pt.SCHEDULE_REFILL, pt.SCHEDULE_WAVEFRONT])
def test_captured_sample_advances_itself(cuda, schedule):
    """rdn_pt_capture: a sample that reads its index from a device counter and
    advances it; three replays equal three samples drawn with host-side counts."""
    import torch

    scene, _, vp, eye = field()
    P = scene.build_product()
    kw = dict(lights=LIGHTS, materials=MATERIALS, traversal=rt.TRAVERSAL_ORDERED_WIDE, schedule=schedule)
    ref = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, **kw)
    for s in (5, 6, 7):
        ref.sample_count = s
        ref.render()
    cap = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, **kw)
    counter = torch.tensor([5], dtype=torch.int32, device="cuda")
    frame = cap.capture(counter)
    for _ in range(3):
        frame()
    torch.cuda.synchronize()
    assert int(counter.item()) == 8
    assert np.array_equal(cap.result(), ref.result())
    assert P.check_errors() == (0, 0)


def test_edge_materials(cuda):
    """Materials at the ends of their ranges: a perfect mirror (roughness 0: GGX's D is 0/0 = NaN, and
    every sample takes the specular lobe), roughness 1, zero reflectance, a black specular colour. NaN
    radiance must match NaN, and the texels (where saturate and the unorm store see it) bit for bit."""
    mats = np.array([pt.metallic_material((1.0, 1.0, 1.0), 0.0, 1.0),
                     pt.metallic_material((0.3, 0.6, 0.9), 1.0, 0.0, 0.0),
                     pt.specular_material((0.7, 0.7, 0.7), 0.3, (0.0, 0.0, 0.0)),
                     pt.metallic_material((0.0, 0.0, 0.0), 0.5, 0.5, 1.0)], pt.MATERIAL_DTYPE)
    for tone in (pt.TONE_MAP_ACES_FILMIC, pt.TONE_MAP_NONE):
        want_img, want_rad, img, rad, rays_o, rays_g = run_pair(
            instanced, lights=LIGHTS, materials=mats, sm_to_material=[0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3],
            tone_map=tone, bg=(0.2, 0.3, 0.4))
        assert np.array_equal(img, want_img) and same_bits(rad, want_rad).all()
        assert rays_g == rays_o
