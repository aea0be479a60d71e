"""Ray-traced ambient occlusion (the reference's feature/ao.rs pipeline):
the fused kernel and the five-group task-graph pipeline against the AO oracle
over several progressive samples. Reference traversal order: every texel
bit-identical; the four-child walk: identical except texels where an
exact-distance tie picks another triangle of the camera ray."""

import numpy as np
import pytest

from helpers import Scene, mat4_cols, orc, rot_z, single_mesh_scene
from rendiation_gb300 import raytracing as rt
from rendiation_gb300 import scenes
from rendiation_gb300 import task_graph as tg

pytestmark = pytest.mark.gpu

W, H = 96, 72
# hammersley(sample, 256) points along the normal for the first samples; later
# ones reach grazing directions, where the rough field occludes
SAMPLES = (150, 200, 250)


def camera(w=W, h=H):
    eye = (0.5, -0.45, 0.75)
    vp = tg.look_at_view_projection_inv(eye, (0.5, 0.5, 0.0), (0, 0, 1), 45.0, w / h, 0.01, 100.0)
    return vp, np.asarray(eye, np.float32)


def vertex_normals(mesh):
    p = mesh.positions.astype(np.float64)
    t = mesh.indices.reshape(-1, 3)
    fn = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, t[:, k], fn)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return n.astype(np.float32)


def run_oracle(scene, samples, normals=None, w=W, h=H):
    S = scene.build_oracle()
    vp, eye = camera(w, h)
    img = np.zeros(w * h, np.uint32)
    for s in samples:
        orc.ao_render(S, vp, eye, w, h, img, sample_count=s, normals=normals, threads=8)
    return img


def run_gpu(scene, samples, traversal, mode, normals=None, block_size=0, speculation=0, w=W, h=H):
    import torch

    P = scene.build_product()
    vp, eye = camera(w, h)
    nt = None if normals is None else torch.from_numpy(normals.reshape(-1)).cuda()
    ao = tg.AmbientOcclusion(P, w, h, vp, eye, traversal=traversal, normals=nt, mode=mode, block_size=block_size,
                             speculation=speculation)
    for s in samples:
        ao.sample_count = s
        ao.render()
    torch.cuda.synchronize()
    flags = P.check_errors()
    img = ao.result().reshape(-1, 4)
    packed = (img[:, 0].astype(np.uint32) | (img[:, 1].astype(np.uint32) << 8) | (img[:, 2].astype(np.uint32) << 16)
              | (img[:, 3].astype(np.uint32) << 24))
    return packed, ao, flags


def field_mesh():
    return scenes.heightfield(48, seed=3, jitter_sigma=0.02)


def field_scene():
    return single_mesh_scene(field_mesh())


@pytest.mark.parametrize("mode", ["fused", "graph"])
@pytest.mark.parametrize("with_normals", [False, True])
def test_reference_order_is_bit_identical_to_the_oracle(cuda, mode, with_normals):
    mesh = field_mesh()
    normals = vertex_normals(mesh) if with_normals else None
    scene = single_mesh_scene(mesh)
    want = run_oracle(scene, SAMPLES, normals)
    got, ao, flags = run_gpu(scene, SAMPLES, rt.TRAVERSAL_REFERENCE, mode, normals)
    assert flags == (0, 0)
    assert np.array_equal(got, want)
    # starting from 0 at sample 150 the bytes encode each pixel's three payloads
    v = want & 0xFF
    assert len(np.unique(v)) >= 3 and 0.005 < (v == 0).mean() < 0.5
    if mode == "graph":
        assert ao.graph.read_back_execution_states().is_empty()
        assert ao.graph.check_errors() == 0


@pytest.mark.parametrize("mode", ["fused", "graph"])
def test_four_child_walk_matches_except_ties(cuda, mode):
    scene = field_scene()
    want = run_oracle(scene, SAMPLES)
    got, _, flags = run_gpu(scene, SAMPLES, rt.TRAVERSAL_ORDERED_WIDE, mode)
    assert flags == (0, 0)
    assert (got == want).mean() > 0.995


@pytest.mark.parametrize("mode", ["fused", "graph"])
@pytest.mark.parametrize("speculation", [4, 16])
def test_leaf_postponement_threshold(cuda, mode, speculation):
    """A lane holding a leaf that keeps descending while more than k lanes of
    its warp look for one only adds node visits: texels stay those of the
    oracle up to exact-distance ties."""
    scene = field_scene()
    want = run_oracle(scene, SAMPLES)
    got, _, flags = run_gpu(scene, SAMPLES, rt.TRAVERSAL_ORDERED_WIDE, mode, speculation=speculation)
    assert flags == (0, 0)
    assert (got == want).mean() > 0.995


@pytest.mark.parametrize("mode", ["fused", "graph"])
@pytest.mark.parametrize("size", [(53, 29), (1, 1), (9, 5)])
def test_ragged_frames(cuda, mode, size):
    """Frames that are not whole 4x8 tiles: the tiles' overhanging pixels
    neither trace nor write; every texel of the frame is the oracle's."""
    w, h = size
    scene = field_scene()
    want = run_oracle(scene, SAMPLES, w=w, h=h)
    got, ao, flags = run_gpu(scene, SAMPLES, rt.TRAVERSAL_REFERENCE, mode, w=w, h=h)
    assert flags == (0, 0)
    assert got.shape == (w * h,)
    assert np.array_equal(got, want)
    if mode == "graph":
        assert ao.graph.read_back_execution_states().is_empty()


def test_graph_equals_fused(cuda):
    scene = field_scene()
    for traversal in (rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE):
        a, _, _ = run_gpu(scene, SAMPLES, traversal, "fused")
        b, _, _ = run_gpu(scene, SAMPLES, traversal, "graph")
        assert np.array_equal(a, b)


@pytest.mark.parametrize("block_size", [32, 64])
def test_block_size_changes_no_texel(cuda, block_size):
    scene = field_scene()
    for traversal in (rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE):
        a, _, _ = run_gpu(scene, SAMPLES, traversal, "fused")
        b, _, flags = run_gpu(scene, SAMPLES, traversal, "fused", block_size=block_size)
        assert flags == (0, 0)
        assert np.array_equal(a, b)


def test_block_size_is_validated(cuda):
    from rendiation_gb300 import native

    P = field_scene().build_product()
    vp, eye = camera()
    ao = tg.AmbientOcclusion(P, W, H, vp, eye, block_size=96)
    with pytest.raises(native.RdnError):
        ao.render()


def test_instanced_scene_with_transforms(cuda):
    a = scenes.heightfield(32, seed=5)
    b = scenes.heightfield(24, seed=6)
    t0 = mat4_cols(rot_z(0.3), (0.6, 0.6, 0.6), (0.1, 0.0, 0.0))
    t1 = mat4_cols(rot_z(-0.2), (-0.5, 0.5, 0.7), (0.9, 0.3, 0.02))  # mirrored
    scene = Scene([[(a.positions, a.indices, 1)], [(b.positions, b.indices, 1)]],
                  [[{"blas": 0, "transform": t0}, {"blas": 1, "transform": t1}]])
    want = run_oracle(scene, SAMPLES)
    got, _, _ = run_gpu(scene, SAMPLES, rt.TRAVERSAL_REFERENCE, "fused")
    assert np.array_equal(got, want)


def test_frozen_after_256_samples(cuda):
    import torch

    scene = field_scene()
    P = scene.build_product()
    vp, eye = camera()
    ao = tg.AmbientOcclusion(P, W, H, vp, eye, traversal=rt.TRAVERSAL_ORDERED_WIDE)
    ao.image.fill_(200)
    ao.sample_count = 256
    before = ao.result().copy()
    ao.render()
    torch.cuda.synchronize()
    assert np.array_equal(ao.result()[..., :3], before[..., :3])
    assert np.all(ao.result()[..., 3] == 255)


@pytest.mark.parametrize("mode", ["fused", "graph"])
def test_captured_frame_advances_its_sample(cuda, mode):
    """rdn_ao_capture: a frame that reads its sample index from a device counter
    and advances it; three replays equal three frames with host-side counts."""
    import torch

    scene = field_scene()
    P = scene.build_product()
    vp, eye = camera()
    ref = tg.AmbientOcclusion(P, W, H, vp, eye, traversal=rt.TRAVERSAL_ORDERED_WIDE, mode=mode)
    for s in SAMPLES:
        ref.sample_count = s
        ref.render()
    cap = tg.AmbientOcclusion(P, W, H, vp, eye, traversal=rt.TRAVERSAL_ORDERED_WIDE, mode=mode)
    counter = torch.tensor([150], dtype=torch.int32, device="cuda")
    frame = cap.capture(counter)
    # the captured frame draws samples 150, 151, 152: compare with those host counts
    ref2 = tg.AmbientOcclusion(P, W, H, vp, eye, traversal=rt.TRAVERSAL_ORDERED_WIDE, mode=mode)
    for s in (150, 151, 152):
        ref2.sample_count = s
        ref2.render()
        frame()
    torch.cuda.synchronize()
    assert int(counter.item()) == 153
    assert np.array_equal(cap.result(), ref2.result())
    assert not np.array_equal(ref2.result(), ref.result())  # the sample indices matter
    assert P.check_errors() == (0, 0)
