"""Camera::update_global_matrix (src/camera.rs:41-51) through the C ABI, entry by entry.

vox_camera_global_matrix is host code of the library (no GPU needed). It is compared with
the oracle's float32 restatement, OPENGL_TO_WGPU_MATRIX * new_perspective * look_at_rh, and
with a float64 numpy restatement of the same published formulas. Both restatements round
differently (the library does not renormalise the up axis of the view, and its products
accumulate in another order), so the tolerance is 2e-6 of the matrix's largest entry, a few
float32 ulps.
"""
import math

import numpy as np
import pytest

TOL = 2e-6


def f64_camera(eye, d, aspect, fovy, zn, zf):
    eye = np.asarray(eye, np.float64)
    z = -np.asarray(d, np.float64)
    z /= np.linalg.norm(z)
    x = np.cross([0.0, 1.0, 0.0], z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    V = np.eye(4)
    V[0, :3], V[1, :3], V[2, :3] = x, y, z
    V[:3, 3] = -V[:3, :3] @ eye
    t = 1.0 / math.tan(fovy / 2.0)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = t / aspect, t
    P[2, 2], P[2, 3], P[3, 2] = (zf + zn) / (zn - zf), 2.0 * zf * zn / (zn - zf), -1.0
    # camera.rs:18-23 written through Matrix4::new, which takes rows
    G = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0.5, 0], [0, 0, 0.5, 1]], np.float64)
    return (G @ P @ V).T.reshape(16)  # column-major


def cases():
    rng = np.random.default_rng(7)
    out = [
        # the reference camera at start-up: eye (0, 0, 1), target direction (0, 0, -1),
        # fov 60 passed through fov.to_degrees() (src/camera.rs:29-36, 47), near 0.01, far 100
        ((0.0, 0.0, 1.0), (0.0, 0.0, -1.0), 16 / 9, float(np.float32(math.degrees(60.0))), 0.01, 100.0),
        # the serving camera of the streaming workload
        ((20.0, 60.0, 0.0), (0.0, -0.342, -0.94), 16 / 9, 1.0471976, 0.1, 416.0),
    ]
    for k in range(300):
        eye = tuple(float(v) for v in rng.uniform(-500, 500, 3).astype(np.float32))
        d = tuple(float(v) for v in rng.normal(size=3).astype(np.float32))
        fovy = float(rng.uniform(0.2, 2.5))
        out.append((eye, d, float(rng.uniform(0.5, 3.0)), fovy, float(rng.uniform(0.01, 1.0)),
                    float(rng.uniform(50.0, 1000.0))))
    return out


def test_camera_matrix_matches_oracle_and_f64(built):
    import voxgpu
    import vox_oracle
    for eye, d, aspect, fovy, zn, zf in cases():
        got = np.asarray(voxgpu.camera_matrix(eye, d, aspect, fovy, zn, zf), np.float32)
        want = vox_oracle.camera_global_matrix(eye, d, aspect, fovy, zn, zf)
        scale = float(np.abs(want).max())
        assert np.abs(got - want).max() <= TOL * scale, (eye, d, got, want)
        ref = f64_camera(eye, d, aspect, fovy, zn, zf)
        assert np.abs(got - ref).max() <= 10 * TOL * max(scale, 1.0), (eye, d)


def test_camera_reference_start_values(built):
    """Hand-derived entries of the reference's first global matrix (eye (0, 0, 1), looking
    down -z, so the view is a translation by -1 in z)."""
    import voxgpu
    fovy = float(np.float32(math.degrees(60.0)))
    m = np.asarray(voxgpu.camera_matrix((0.0, 0.0, 1.0), (0.0, 0.0, -1.0), 16 / 9, fovy, 0.01,
                                        100.0), np.float32).reshape(4, 4).T  # row-major view
    t = np.float32(1.0) / np.tan(np.float32(fovy) / np.float32(2.0))
    assert m[1, 1] == pytest.approx(float(t), rel=1e-6)
    assert m[0, 0] == pytest.approx(float(t) / (16 / 9), rel=1e-6)
    assert m[3, 2] == pytest.approx(0.5 * (100.01 / (0.01 - 100.0)) - 1.0, rel=1e-5)
    assert m[0, 1] == 0.0 and m[1, 0] == 0.0


def test_camera_rejects_degenerate_input(built):
    import voxgpu
    with pytest.raises(voxgpu.VoxError):
        voxgpu.camera_matrix((0, 0, 0), (0, 0, 0))
    with pytest.raises(voxgpu.VoxError):
        voxgpu.camera_matrix((0, 0, 0), (0, 1, 0))  # direction parallel to up
