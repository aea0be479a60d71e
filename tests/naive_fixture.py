"""The reference's own ray-tracing test scene, restated in FP32.

The reference's BVH tests (shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/test.rs)
share one fixture, `init_default_acceleration_structure` (test.rs:9-225): three BLAS (a UV sphere
tessellated 32x16, a torus tessellated 32x8, an indexed 24-vertex cube) and five TLAS built from
them, traced by `test_cpu_triangle` / `test_gpu_triangle_naive` (test.rs:233-372) with a 256x256,
90-degree pinhole camera at the origin, back faces culled. This module rebuilds that fixture with
the same formulas and the same FP32 operation order:

* tessellation: content/mesh/generator/src/builder/mod.rs:73-128 (`triangulate_parametric`): an
  (nu+1) x (nv+1) vertex grid, u outer, v inner; cell (u, v) gives triangles (a, c, b) and (b, c, d)
  with a = (u, v), b = (u, v+1), c = (u+1, v), d = (u+1, v+1).
* sphere: content/mesh/generator/src/builtin.rs:85-116 with the default parameters, over
  primitive.rs `UVSphere` and combination.rs `ParametricSurfaceRangeMapping`. The range mapping
  interpolates both coordinates with the u range (combination.rs:35-37); that is restated as is.
* torus: builtin.rs:9-21, a unit circle scaled to the radius, embedded in the XY plane and swept
  by a circle of the tube radius (combination.rs `FixedSweepSurface`). The path's normal and
  tangent come from the finite-difference defaults of parametric.rs:10-38 (EPS = 1e-4).
* cube: the 24-vertex, 12-triangle table of test.rs:79-96, written here from its corner names.
* transforms: math/algebra/src/mat/mat4.rs (`Mat4::new` fills columns a, b, c, d in turn,
  `translate` / `scale` / `rotate_x|y|z`, products summed left to right).
* camera: test.rs:258-264, x = (i + 0.5) / W * 2 - 1, y = 1 - (j + 0.5) / H * 2, direction the
  normalised (x, y, -1).

Sine and cosine are the FP32 roundings of the double-precision values. The reference calls the
platform's FP32 `sin_cos`, which may differ from them by one ulp for some angles. Parity compares
the product with the oracle on these arrays, so that difference does not enter it.
"""

from __future__ import annotations

import math

import numpy as np

from helpers import Scene, scenes

F = np.float32
PI = F(math.pi)          # f32::PI()
EPS = F(1e-4)            # parametric.rs:3
ONE, ZERO, TWO, HALF = F(1), F(0), F(2), F(0.5)

W = H = 256              # test.rs:235-236
FAR = 100.0              # test.rs:237
PRIMITIVE_IDX_MAX = 12   # test.rs:240
TEST_TLAS_IDX = 4        # test.rs:6
CPU_TEST_RANGE = (0.0, FAR)     # test.rs:250
GPU_TEST_RANGE = (0.01, FAR)    # test.rs:371


def sin_cos(x):
    x = float(x)
    return F(math.sin(x)), F(math.cos(x))


# ---- FP32 vector / matrix arithmetic in the reference's operation order ----

def v_sub(a, b):
    return tuple(F(x - y) for x, y in zip(a, b))


def v_scale(a, s):
    return tuple(F(x * s) for x in a)


def v_dot(a, b):
    acc = F(a[0] * b[0])
    for x, y in zip(a[1:], b[1:]):
        acc = F(acc + F(x * y))
    return acc


def v_cross(a, b):
    return (F(F(a[1] * b[2]) - F(a[2] * b[1])), F(F(a[2] * b[0]) - F(a[0] * b[2])),
            F(F(a[0] * b[1]) - F(a[1] * b[0])))


def v_normalize(a):
    """InnerProductSpace::normalize (vec/dimension.rs:98-105): a * (1 / sqrt(|a|^2)) when |a|^2 > 0."""
    m = v_dot(a, a)
    if m > ZERO:
        return v_scale(a, F(ONE / np.sqrt(m)))
    return a


def lerp(a, b, t):
    """interpolation.rs:8: a * (1 - t) + b * t."""
    return F(F(a * F(ONE - t)) + F(b * t))


def mat4(*m):
    """Mat4::new: sixteen values, columns a, b, c, d in turn (the memory order of the reference)."""
    return tuple(F(x) for x in m)


def mat4_mul(a, m):
    """Mat4 * Mat4 (mat4.rs:171-200): column k of the product is A applied to column k of m."""
    out = []
    for col in range(4):
        mc = m[4 * col:4 * col + 4]
        for row in range(4):
            acc = F(a[row] * mc[0])
            for k in range(1, 4):
                acc = F(acc + F(a[4 * k + row] * mc[k]))
            out.append(acc)
    return tuple(out)


def mat4_apply(m, p):
    """Mat4 * Vec3 (mat4.rs:134-145): (x, y, z, 1) through the matrix, then divided by w."""
    v = (p[0], p[1], p[2], ONE)
    r = []
    for row in range(4):
        acc = F(v[0] * m[row])
        for k in range(1, 4):
            acc = F(acc + F(v[k] * m[4 * k + row]))
        r.append(acc)
    return (F(r[0] / r[3]), F(r[1] / r[3]), F(r[2] / r[3]))


def translate(x, y, z):
    return mat4(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, x, y, z, 1)


def scale(x, y, z):
    return mat4(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1)


def rotate_x(theta):
    s, c = sin_cos(F(theta))
    return mat4(1, 0, 0, 0, 0, c, s, 0, 0, -s, c, 0, 0, 0, 0, 1)


def rotate_y(theta):
    s, c = sin_cos(F(theta))
    return mat4(c, 0, -s, 0, 0, 1, 0, 0, s, 0, c, 0, 0, 0, 0, 1)


def rotate_z(theta):
    s, c = sin_cos(F(theta))
    return mat4(c, s, 0, 0, -s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)


def chain(*ms):
    out = ms[0]
    for m in ms[1:]:
        out = mat4_mul(out, m)
    return out


def mat3_scale_apply(s, p):
    """Mat3::scale(Vec2::splat(s)) * Vec2 (mat3.rs:75-110, 285-297): homogeneous, divided by z."""
    x = F(F(F(p[0] * s) + F(p[1] * ZERO)) + F(ONE * ZERO))
    y = F(F(F(p[0] * ZERO) + F(p[1] * s)) + F(ONE * ZERO))
    z = F(F(F(p[0] * ZERO) + F(p[1] * ZERO)) + F(ONE * ONE))
    return (F(x / z), F(y / z))


# ---- parametric surfaces ----

def unit_circle(t):
    """primitive.rs UnitCircle: (cos, sin) of t * pi * 2."""
    s, c = sin_cos(F(F(t * PI) * TWO))
    return (c, s)


def sphere_position(u, v):
    """SphereMeshParameter::default().make_surface(): UVSphere scaled by 1, its parameters
    mapped through [phi_start, phi_start + phi_length] / (2 pi) (for both coordinates, as the
    reference's range mapping does)."""
    to_u = F(ONE / F(TWO * PI))
    u0 = F(ZERO * to_u)
    u1 = F(F(ZERO + F(PI * TWO)) * to_u)
    mu, mv = lerp(u0, u1, u), lerp(u0, u1, v)
    us, uc = sin_cos(F(F(mu * PI) * TWO))
    vs, vc = sin_cos(F(mv * PI))
    p = (F(uc * vs), vc, F(us * vs))
    return mat4_apply(scale(1, 1, 1), p)


def plane_normal_dir(p2):
    """ParametricSurface::normal_dir default (parametric.rs:10-27) on ParametricPlane."""
    x, y = p2
    if F(x + EPS) >= ONE:
        x = F(ONE - EPS)
    if F(y + EPS) >= ONE:
        y = F(ONE - EPS)
    p = (x, y, ZERO)
    pu = (F(x + EPS), y, ZERO)
    pv = (x, F(y + EPS), ZERO)
    return v_cross(v_sub(pu, p), v_sub(pv, p))


def torus_surface(radius, tube_radius):
    radius, tube_radius = F(radius), F(tube_radius)

    def path_position(t):
        c = mat3_scale_apply(radius, unit_circle(t))
        return (c[0], c[1], ZERO)

    def position(u, v):
        cs = mat3_scale_apply(tube_radius, unit_circle(v))
        point = (cs[0], cs[1], ZERO)
        origin = path_position(u)
        normal = v_normalize(plane_normal_dir(mat3_scale_apply(radius, unit_circle(u))))
        tangent = v_normalize(v_sub(path_position(F(u + EPS)), origin))   # parametric.rs:35-39
        right = v_cross(tangent, normal)
        # Mat4::from_orth_basis_and_position(forward = tangent, up = normal, origin), mat4.rs:254-264
        m = mat4(*right, 0, *normal, 0, *tangent, 0, *origin, 1)
        return mat4_apply(m, point)

    return position


def triangulate(surface, nu: int, nv: int) -> scenes.Mesh:
    u_step, v_step = F(ONE / F(nu)), F(ONE / F(nv))
    verts = [surface(F(F(u) * u_step), F(F(v) * v_step)) for u in range(nu + 1) for v in range(nv + 1)]
    idx = []
    for u in range(nu):
        for v in range(nv):
            a = v + (nv + 1) * u
            b, c = a + 1, a + nv + 1
            idx += [a, c, b, b, c, c + 1]
    return scenes.Mesh(np.array(verts, np.float32).reshape(-1, 3), np.array(idx, np.uint32))


def cube() -> scenes.Mesh:
    """The unit cube of test.rs:79-96: four vertices per face, faces front, right, top, left,
    bottom, back, each face two triangles (0, 1, 2), (2, 3, 0) of its four vertices."""
    corner = {0: (1, 1, 1), 1: (-1, 1, 1), 2: (-1, -1, 1), 3: (1, -1, 1),
              4: (1, -1, -1), 5: (1, 1, -1), 6: (-1, 1, -1), 7: (-1, -1, -1)}
    faces = [(0, 1, 2, 3), (0, 3, 4, 5), (0, 5, 6, 1), (1, 6, 7, 2), (7, 4, 3, 2), (4, 7, 6, 5)]
    pos = np.array([[0.5 * c for c in corner[k]] for f in faces for k in f], np.float32)
    idx = np.array([4 * f + k for f in range(6) for k in (0, 1, 2, 2, 3, 0)], np.uint32)
    return scenes.Mesh(pos, idx)


def sphere_mesh() -> scenes.Mesh:
    return triangulate(sphere_position, 32, 16)


def torus_mesh() -> scenes.Mesh:
    return triangulate(torus_surface(1.0, 0.2), 32, 8)


# ---- the five TLAS (test.rs:136-219) ----

SPHERE, TORUS, CUBE = 0, 1, 2   # BLAS handles in creation order


def tlas_instances() -> list[list[tuple[int, tuple]]]:
    t0 = [(CUBE, translate(F(F(i) * F(1.5)), F(F(j) * F(1.5)), -10.0)) for i in range(-2, 3) for j in range(-2, 3)]
    t0.append((CUBE, chain(translate(0.0, 4.5, -10.0), scale(5.0, 1.0, 1.0))))
    t0.append((CUBE, chain(translate(0.0, -4.5, -10.0), rotate_y(PI), scale(5.0, 1.0, 1.0))))
    t0.append((CUBE, chain(translate(4.5, -4.5, -10.0), rotate_y(F(PI * HALF)), scale(5.0, 1.0, 1.0))))
    t0.append((CUBE, chain(translate(-4.5, -4.5, -10.0), rotate_y(F(PI * F(-0.5))), scale(5.0, 1.0, 1.0))))
    t1 = []
    for i in range(6):
        angle = F(F(F(F(i) / F(6.0)) * PI) * TWO)
        s, c = sin_cos(angle)
        t1.append((CUBE, chain(translate(F(s * F(4)), F(c * F(4)), -5.0), rotate_z(F(-angle)), scale(3.0, 0.5, 0.5))))
    t2 = [(TORUS, chain(translate(0.0, 0.0, -10.0), scale(5.0, 5.0, 5.0), rotate_x(-0.5)))]
    t3 = [(CUBE, translate(F(F(i) * F(1.5)), F(F(j) * F(1.5)), F(F(-8.0) + F(F(k) * F(1.5)))))
          for i in range(-2, 3) for j in range(-2, 3) for k in range(-2, 3)]
    t4 = [(SPHERE, chain(translate(0.0, 0.0, -10.0), scale(5.0, 5.0, 5.0)))]
    return [t0, t1, t2, t3, t4]


def meshes() -> list[scenes.Mesh]:
    return [sphere_mesh(), torus_mesh(), cube()]


def make_scene(mesh_list=None, transforms=None, bind=None) -> Scene:
    """All five TLAS bound in order unless `bind` says otherwise (the reference binds TLAS 4 alone).
    Geometry flags opaque; instances with mask 0xFF, custom index 0, no flags (test.rs:115-127)."""
    mesh_list = meshes() if mesh_list is None else mesh_list
    inst = tlas_instances()
    if transforms is not None:
        it = iter(np.asarray(transforms, np.float32).reshape(-1, 16))
        inst = [[(b, tuple(next(it))) for b, _ in t] for t in inst]
    blas = [[(m.positions, m.indices, 1)] for m in mesh_list]
    tlas = [[{"blas": b, "transform": np.asarray(m, np.float32), "mask": 0xFF} for b, m in t] for t in inst]
    return Scene(blas, tlas, bind=bind)


def all_transforms() -> np.ndarray:
    return np.array([m for t in tlas_instances() for _, m in t], np.float32)


def camera_rays(tmin: float, tmax: float = FAR) -> np.ndarray:
    """The 256x256 rays of test.rs:258-264, row j outer, column i inner."""
    j, i = np.meshgrid(np.arange(H, dtype=np.float32), np.arange(W, dtype=np.float32), indexing="ij")
    x = (i + HALF) / F(W) * TWO - ONE
    y = ONE - (j + HALF) / F(H) * TWO
    z = np.full_like(x, -1.0)
    m = x * x + y * y + z * z
    inv = ONE / np.sqrt(m)
    dirs = np.stack([x * inv, y * inv, z * inv], -1).reshape(-1, 3).astype(np.float32)
    return scenes.make_rays(np.zeros_like(dirs), dirs, tmin, tmax)


def id_image(prim: np.ndarray, miss: int) -> np.ndarray:
    """test.rs:266-270: primitive % 12 + 1 where a ray hit, 0 elsewhere (the P2 image's values)."""
    p = np.asarray(prim, np.uint32)
    return np.where(p == np.uint32(miss), 0, p % PRIMITIVE_IDX_MAX + 1).astype(np.uint8).reshape(H, W)
