"""The C oracle's culling against a second, independent restatement of the reference's
rule in plain Python (src/chunk.rs:59-245), on seeded random chunks and neighbours.

For every solid voxel in y -> z -> x order the reference emits, in this order, LEFT
(-x), RIGHT (+x), BACK (-z), FRONT (+z), DOWN (-y), UP (+y) when the voxel on that side is
air. On a lateral border the side voxel comes from the loaded neighbour chunk (its
opposite border), and a neighbour that is not loaded counts as air; on the y borders the
face is always emitted (reference mode), or (full-6 mode, not a reference behaviour) the
-y / +y neighbours decide like the lateral ones."""
import numpy as np
import pytest

AIR = 2


def restated_faces(n, cubes, adj, full6):
    def solid(c, x, y, z):
        return c[x + n * z + n * n * y] != AIR

    # (dx, dy, dz, neighbour slot, coordinate in the neighbour) per direction L R Bk F D U
    out = []
    for y in range(n):
        for z in range(n):
            for x in range(n):
                if not solid(cubes, x, y, z):
                    continue
                sides = (
                    (x > 0, (x - 1, y, z), 0, (n - 1, y, z)),
                    (x < n - 1, (x + 1, y, z), 1, (0, y, z)),
                    (z > 0, (x, y, z - 1), 2, (x, y, n - 1)),
                    (z < n - 1, (x, y, z + 1), 3, (x, y, 0)),
                    (y > 0, (x, y - 1, z), 4, (x, n - 1, z)),
                    (y < n - 1, (x, y + 1, z), 5, (x, 0, z)),
                )
                for d, (inside, p, slot, q) in enumerate(sides):
                    if inside:
                        exposed = not solid(cubes, *p)
                    elif slot >= 4 and not full6:
                        exposed = True  # y borders: always emitted
                    elif adj[slot] is None:
                        exposed = True  # neighbour not loaded: counts as air
                    else:
                        exposed = not solid(adj[slot], *q)
                    if exposed:
                        out.append((x, y, z, d))
    return out


@pytest.mark.parametrize("case", range(12))
def test_culling_matches_an_independent_restatement(oracle, case):
    rng = np.random.default_rng(500 + case)
    n = 8
    full6 = case % 2 == 1
    density = [0.1, 0.5, 0.9][case % 3]

    def chunk():
        return np.where(rng.random(n ** 3) < density, 0, AIR).astype(np.uint8)

    cubes = chunk()
    adj = [chunk() if rng.random() < 0.6 else None for _ in range(6)]
    want = restated_faces(n, cubes, adj, full6)
    got = oracle.cull_faces(n, 1 if full6 else 0, cubes, adj)
    assert [tuple(int(v) for v in f) for f in got.tolist()] == want
