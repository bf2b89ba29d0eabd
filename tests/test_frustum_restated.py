"""The oracle's frustum (src/frustum_culling.rs:16-85) against an independent float32
restatement: Gribb-Hartmann planes from the column-major global matrix in the order near,
far, left, right, top, bottom, and a chunk visible iff one of its 8 corners is on the
inner side of all six planes (the reference's corner-only test), with every dot product
evaluated left to right in float32."""
import numpy as np
import pytest

F = np.float32


def restated_planes(m):
    at = lambda c, r: F(m[4 * c + r])  # column c, row r
    rows = [(2, 1), (2, -1), (0, 1), (0, -1), (1, -1), (1, 1)]  # near far left right top bottom
    out = []
    for k, sign in rows:
        out += [at(c, 3) + at(c, k) if sign > 0 else at(c, 3) - at(c, k) for c in range(4)]
    return np.array(out, np.float32)


def restated_contains(planes, coord, extent):
    e = F(extent)
    x0, y0, z0 = (F(v * extent) for v in coord)
    for dx in (F(0), e):
        for dy in (F(0), e):
            for dz in (F(0), e):
                x, y, z = x0 + dx, y0 + dy, z0 + dz
                inside = True
                for i in range(6):
                    a, b, c, d = planes[4 * i: 4 * i + 4]
                    if ((a * x + b * y) + c * z) + d < F(0):
                        inside = False
                        break
                if inside:
                    return True
    return False


def matrices(vox, rng):
    ms = [np.asarray(vox.camera_matrix(eye, d), np.float32)
          for eye, d in [((0, 60, 0), (1, -0.3, 0)), ((100, 40, -50), (-0.2, -0.1, 1)),
                         ((-30, 80, 20), (0.5, -0.5, -0.5))]]
    ms += [rng.standard_normal(16).astype(np.float32) for _ in range(5)]
    return ms


@pytest.mark.parametrize("extent", [16, 32])
def test_frustum_matches_an_independent_restatement(vox, oracle, extent):
    rng = np.random.default_rng(extent)
    seen = set()
    for m in matrices(vox, rng):
        want_planes = restated_planes(m)
        got_planes = oracle.frustum_planes(m)
        assert np.array_equal(got_planes.view(np.uint32), want_planes.view(np.uint32))
        for coord in rng.integers(-12, 12, (200, 3)):
            c = tuple(int(v) for v in coord)
            want = restated_contains(want_planes, c, extent)
            assert oracle.frustum_contains(got_planes, c, extent) == want, (c, extent)
            seen.add(want)
    assert seen == {True, False}
