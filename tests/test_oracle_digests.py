"""The full-size parity checker on the CPU: or_gen_mesh_digests (the oracle chunk by chunk
on host threads, as the full-size GPU tests use it) against or_gen_mesh_batch's bytes
digested per chunk, and the digests' sensitivity to a single changed byte."""
import numpy as np
import pytest


def _case(vox, name):
    wl = vox.workload(name)
    if name == "density":
        coords = vox.grid_coords(range(4, 7), range(7, 10), range(4, 7))
    elif name == "stress":
        coords = list(wl.coords[:4])
    else:
        coords = list(wl.coords[:128])
    masks = None if wl.isolated else vox.neighbour_masks(coords)
    return wl, coords, masks


@pytest.mark.parametrize("name", ["plain", "heightmap", "density", "stress"])
@pytest.mark.parametrize("layout", [0, 1])
def test_chunk_digests_equal_the_batch_bytes(vox, oracle, name, layout):
    wl, coords, masks = _case(vox, name)
    cfg = wl.config(layout=layout)
    base = 1000 if name == "stress" else 0
    o0, o1, offs = oracle.gen_mesh_batch(cfg, coords, masks, base)
    b0, b1 = oracle.bytes_per_face(layout)
    want = oracle.chunk_digests(o0, o1, offs, b0, b1)
    for threads in (1, 3):
        counts, dig = oracle.gen_mesh_digests(cfg, coords, masks, base, nthreads=threads)
        assert np.array_equal(counts, np.diff(offs)), (name, threads)
        assert np.array_equal(dig, want), (name, threads)
    # one chunk's digest is the digest of its own byte ranges
    k = int(np.argmax(np.diff(offs)))
    lo, hi = int(offs[k]), int(offs[k + 1])
    assert oracle.digest(o0[lo * b0:hi * b0]) == int(want[k, 0])
    if b1:
        assert oracle.digest(o1[lo * b1:hi * b1]) == int(want[k, 1])


def test_a_changed_byte_changes_exactly_its_chunks_digest(vox, oracle):
    wl, coords, masks = _case(vox, "heightmap")
    cfg = wl.config()
    o0, o1, offs = oracle.gen_mesh_batch(cfg, coords, masks)
    want = oracle.chunk_digests(o0, o1, offs, 96, 24)
    rng = np.random.default_rng(5)
    nonempty = np.flatnonzero(np.diff(offs))
    for _ in range(20):
        k = int(rng.choice(nonempty))
        which = int(rng.integers(2))
        buf, b = (o0, 96) if which == 0 else (o1, 24)
        at = int(rng.integers(int(offs[k]) * b, int(offs[k + 1]) * b))
        bad = buf.copy()
        bad[at] ^= np.uint8(1 << int(rng.integers(8)))
        got = oracle.chunk_digests(bad if which == 0 else o0, bad if which == 1 else o1, offs, 96, 24)
        diff = np.argwhere(got != want)
        assert diff.tolist() == [[k, which]]
