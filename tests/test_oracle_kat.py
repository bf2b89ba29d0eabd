"""Known-answer tests of the CPU oracle, derived by hand from the reference's rules.

The reference (Blatko1/wgpu-voxel-engine) ships no tests or golden vectors, so the
oracle is pinned here against answers that follow directly from its source:
src/chunk.rs:59-245 (culling and emission order), src/quad.rs:14-89 (rotations, quad
vertices and indices), src/frustum_culling.rs:16-85 (planes and the AABB test).
"""
import itertools
import struct

import numpy as np
import pytest

AIR, GRASS = 2, 0
L, R, BK, F, D, U = range(6)


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def cubes_all(n, v):
    return np.full(n * n * n, v, np.uint8)


def idx(n, x, y, z):
    return x + n * z + n * n * y


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_all_air_has_no_faces(oracle, n):
    assert len(oracle.cull_faces(n, 0, cubes_all(n, AIR))) == 0


@pytest.mark.parametrize("n", [8, 32])
def test_single_voxel_emits_six_faces_in_reference_order(oracle, n):
    c = cubes_all(n, AIR)
    c[idx(n, 3, 4, 5)] = GRASS
    f = oracle.cull_faces(n, 0, c)
    # chunk.rs:76-240: LEFT, RIGHT, BACK, FRONT, DOWN, UP for one voxel.
    assert f.tolist() == [[3, 4, 5, d] for d in range(6)]


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_full_chunk_without_neighbours(oracle, n):
    # Every border face is emitted: 6 N^2 faces.
    assert len(oracle.cull_faces(n, 0, cubes_all(n, GRASS))) == 6 * n * n


@pytest.mark.parametrize("n", [8, 32])
def test_full_chunk_with_solid_lateral_neighbours(oracle, n):
    full = cubes_all(n, GRASS)
    f = oracle.cull_faces(n, 0, full, [full] * 4)
    # Only the y borders remain (chunk.rs:216-221, 234-239): N^2 DOWN + N^2 UP.
    assert len(f) == 2 * n * n
    assert set(f[:, 3].tolist()) == {D, U}
    # The -y/+y neighbours are ignored in reference mode...
    assert len(oracle.cull_faces(n, 0, full, [full] * 6)) == 2 * n * n
    # ...and consulted in the full 6-neighbour mode.
    assert len(oracle.cull_faces(n, 1, full, [full] * 6)) == 0


@pytest.mark.parametrize("n", [8, 16])
def test_checkerboard(oracle, n):
    c = np.array([GRASS if (x + y + z) % 2 == 0 else AIR
                  for y in range(n) for z in range(n) for x in range(n)], np.uint8)
    # every solid voxel is isolated: 6 faces each, N^3/2 solid voxels
    assert len(oracle.cull_faces(n, 0, c)) == 3 * n ** 3


def test_lateral_neighbour_decides_border_face(oracle):
    n = 8
    c = cubes_all(n, AIR)
    c[idx(n, 0, 2, 2)] = GRASS
    nb = cubes_all(n, AIR)
    f = oracle.cull_faces(n, 0, c, [nb, None, None, None])
    assert [L] == [d for (_, _, _, d) in f.tolist() if d == L]
    nb[idx(n, n - 1, 2, 2)] = GRASS  # the -x neighbour's x = N-1 voxel is solid
    f = oracle.cull_faces(n, 0, c, [nb, None, None, None])
    assert L not in f[:, 3].tolist()
    # +z: chunk.rs:186-196 reads the +z neighbour's z = 0 row
    c2 = cubes_all(n, AIR)
    c2[idx(n, 4, 1, n - 1)] = GRASS
    nz = cubes_all(n, AIR)
    nz[idx(n, 4, 1, 0)] = GRASS
    f = oracle.cull_faces(n, 0, c2, [None, None, None, nz])
    assert F not in f[:, 3].tolist() and len(f) == 5


def test_emission_order_is_y_then_z_then_x(oracle):
    n = 8
    c = cubes_all(n, AIR)
    pts = [(5, 0, 0), (1, 0, 3), (2, 1, 0), (0, 0, 0)]
    for p in pts:
        c[idx(n, *p)] = GRASS
    f = oracle.cull_faces(n, 0, c)
    voxels = [tuple(v[:3]) for v in f[::6]]
    assert voxels == sorted(voxels, key=lambda v: (v[1], v[2], v[0]))


def test_splitmix64_and_permutation(oracle):
    import ctypes
    s = ctypes.c_uint64(0)
    L_ = oracle.load()
    # splitmix64 seeded with 0: first output of the published generator.
    assert L_.or_splitmix64_next(ctypes.byref(s)) == 0xE220A8397B1DCDAF
    p = oracle.perm(42)
    assert sorted(p[:256].tolist()) == list(range(256))
    assert (p[:256] == p[256:]).all()
    assert not (oracle.perm(42) == oracle.perm(7)).all()


def test_noise_lattice_zero_and_slice(oracle):
    L_ = oracle.load()
    p = oracle.perm(1234)
    pa = int(p.ctypes.data)
    for x, y, z in itertools.product([-3.0, 0.0, 5.0], repeat=3):
        assert L_.or_noise3_f32(pa, x, y, z) == 0.0  # gradient noise vanishes on the lattice
    rng = np.random.default_rng(0)
    for _ in range(200):
        x, y = rng.uniform(-300, 300, 2).astype(np.float32)
        a = L_.or_noise2_f32(pa, float(x), float(y))
        b = L_.or_noise3_f32(pa, float(x), float(y), 0.0)
        assert a == b  # noise2 is the z = 0 slice of noise3
        assert abs(a - L_.or_noise2_f64(pa, float(x), float(y))) < 1e-5
        assert -1.5 < a < 1.5


def test_face_rotations(oracle):
    # f32 to_radians(90) = 1.5707964 and glibc sinf/cosf of it, as in quad.rs:19-38.
    cos_half_pi = -4.37113883e-08
    r_left = oracle.face_rotation(L)     # pitch -90
    r_right = oracle.face_rotation(R)    # pitch 90
    r_back = oracle.face_rotation(BK)    # pitch 180
    r_front = oracle.face_rotation(F)    # identity
    r_down = oracle.face_rotation(D)     # roll 90
    r_up = oracle.face_rotation(U)       # roll -90
    assert (r_front == np.eye(3, dtype=np.float32)).all()
    assert f32_bits(r_right[0, 0]) == f32_bits(np.float32(cos_half_pi))
    assert r_right[0, 2] == 1.0 and r_right[2, 0] == -1.0
    assert r_left[0, 2] == -1.0 and r_left[2, 0] == 1.0
    assert r_back[0, 0] == -1.0 and r_back[2, 2] == -1.0
    assert f32_bits(r_back[0, 2]) == f32_bits(np.float32(-8.74227766e-08))
    assert r_down[1, 2] == -1.0 and r_down[2, 1] == 1.0
    assert r_up[1, 2] == 1.0 and r_up[2, 1] == -1.0
    for r in (r_left, r_right, r_back, r_down, r_up):
        assert np.allclose(r @ r.T, np.eye(3), atol=1e-6)


def test_instance_and_vertex_records(oracle):
    import ctypes
    L_ = oracle.load()
    rec = np.zeros(17, np.uint32)
    L_.or_instance_raw(F, 3, -4, 5, 7, int(rec.ctypes.data))
    m = rec[:16].view(np.float32).reshape(4, 4)  # t_matrix[col][row]
    assert m[3, :3].tolist() == [3.0, -4.0, 5.0] and m[3, 3] == 1.0
    assert (m[:3, :3] == np.eye(3)).all()
    assert rec[16] == 7
    v = np.zeros(24, np.uint32)
    ix = np.zeros(6, np.uint32)
    L_.or_face_vertices(F, 0, 0, 0, 2, int(v.ctypes.data), int(ix.ctypes.data))
    vf = v.view(np.float32).reshape(4, 6)
    # FRONT face = quad::VERTICES unrotated (src/quad.rs:66-87)
    assert vf[:, :3].tolist() == [[-0.5, 0.5, 0.5], [0.5, 0.5, 0.5], [-0.5, -0.5, 0.5],
                                  [0.5, -0.5, 0.5]]
    assert vf[:, 3:5].tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    assert v.reshape(4, 6)[:, 5].tolist() == [3] * 4  # slot of FRONT
    assert ix.tolist() == [8, 10, 9, 11, 9, 10]  # 4*2 + quad::INDICES
    # UP face of voxel (0, 0, 0): the quad lies on y = +0.5 (roll -90: z -> y)
    L_.or_face_vertices(U, 0, 0, 0, 0, int(v.ctypes.data), int(ix.ctypes.data))
    assert np.allclose(v.view(np.float32).reshape(4, 6)[:, 1], 0.5)
    assert v.reshape(4, 6)[0, 5] == 4
    _ = ctypes


def perspective_look(eye, fwd, aspect=16 / 9, fovy=1.2, near=0.01, far=100.0):
    f = 1.0 / np.tan(fovy / 2)
    P = np.array([[f / aspect, 0, 0, 0], [0, f, 0, 0],
                  [0, 0, (far + near) / (near - far), 2 * far * near / (near - far)],
                  [0, 0, -1, 0]], np.float64)
    fwd = np.asarray(fwd, np.float64) / np.linalg.norm(fwd)
    up = np.array([0, 1, 0.0])
    s = np.cross(fwd, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, fwd)
    V = np.eye(4)
    V[0, :3], V[1, :3], V[2, :3] = s, u, -fwd
    V[:3, 3] = -V[:3, :3] @ np.asarray(eye, np.float64)
    G = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0.5, 0.5], [0, 0, 0, 1.0]])
    return (G @ P @ V).astype(np.float32)


def test_frustum(oracle):
    M = perspective_look([16, 16, 16], [0, 0, -1])
    planes = oracle.frustum_planes(M.T.reshape(16))  # column-major
    assert oracle.frustum_contains(planes, (0, 0, -1), 32)       # straight ahead
    assert not oracle.frustum_contains(planes, (0, 0, 3), 32)    # behind the camera
    assert not oracle.frustum_contains(planes, (0, 0, -40), 32)  # beyond the far plane
    # frustum_culling.rs:27-39 tests only the 8 corners: the chunk around the eye has no
    # corner inside the view volume and is reported invisible (a reference quirk).
    assert not oracle.frustum_contains(planes, (0, 0, 0), 32)


def _one_face(slot, order=(0, 2, 1, 3, 1, 2), z=0.5):
    """One vertex-layout face: quad::VERTICES at depth z (NDC), texture slot `slot`."""
    pos = [(-0.5, 0.5), (0.5, 0.5), (-0.5, -0.5), (0.5, -0.5)]
    uv = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0)]
    v = b"".join(np.array([p[0], p[1], z, t[0], t[1]], np.float32).tobytes()
                 + np.array([slot], np.uint32).tobytes() for p, t in zip(pos, uv))
    return v, np.array(order, np.uint32).tobytes()


def test_raster_single_face_known_pixels(oracle):
    """Identity matrix, one front face covering NDC [-0.5, 0.5]^2 on an 8x8 image: pixels
    2..5 in x and y carry the checkered top colour, everything else the clear colour."""
    ident = np.eye(4, dtype=np.float32).reshape(16)
    tex = (0, 0, 0, 0, 2, 1)
    v, i = _one_face(4)
    img = oracle.raster(ident, v, i, 1, 8, 8, tex)
    clear = (26, 51, 77, 255)
    light, dark = (77, 179, 64, 255), (65, 152, 54, 255)
    for py in range(8):
        for px in range(8):
            got = tuple(int(c) for c in img[py, px])
            if 2 <= px <= 5 and 2 <= py <= 5:
                want = light if ((px - 2) + (py - 2)) % 2 == 0 else dark
            else:
                want = clear
            assert got == want, (px, py, got, want)
    # the same face wound the other way is a back face: culled
    vb, ib = _one_face(4, order=(0, 1, 2, 3, 2, 1))
    img = oracle.raster(ident, vb, ib, 1, 8, 8, tex)
    assert (img.reshape(-1, 4) == np.array(clear, np.uint8)).all()


def test_raster_depth_less_first_drawn_wins(oracle):
    """Two faces at the same depth: the first drawn keeps the pixels (depth test Less);
    a nearer face drawn later replaces them."""
    ident = np.eye(4, dtype=np.float32).reshape(16)
    tex = (0, 0, 0, 0, 2, 1)
    v_top, i_top = _one_face(4, z=0.5)
    v_side, _ = _one_face(0, z=0.5)
    i2 = np.array([0, 2, 1, 3, 1, 2, 4, 6, 5, 7, 5, 6], np.uint32).tobytes()
    img = oracle.raster(ident, v_top + v_side, i2, 2, 8, 8, tex)
    assert tuple(int(c) for c in img[2, 2]) == (77, 179, 64, 255)   # top colour (first)
    v_near, _ = _one_face(0, z=0.25)
    img = oracle.raster(ident, v_top + v_near, i2, 2, 8, 8, tex)
    assert tuple(int(c) for c in img[2, 2]) == (115, 140, 64, 255)  # side colour (nearer)
