"""The CPU baseline (or_baseline_run: the reference's pool work, Chunk::new then create_mesh
per chunk, on host threads) does the same work as the oracle's batch path: with masks that
mark exactly the neighbours inside the batch (the World.chunks lookup), its face total
equals the batch's, for every generator, both layouts and both cull modes, on one thread
and on several."""
import pytest


def _cases(vox):
    hm = vox.workload("heightmap")
    yield "heightmap", hm, list(hm.coords[:256])
    pl = vox.workload("plain")
    yield "plain", pl, list(pl.coords)
    de = vox.workload("density")
    yield "density", de, vox.grid_coords(range(4, 8), range(7, 10), range(4, 8))
    st = vox.workload("stress")
    yield "stress", st, list(st.coords[:6])


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("cull", [0, 1])
def test_baseline_faces_equal_the_batch_oracle(vox, oracle, layout, cull):
    for name, wl, coords in _cases(vox):
        cfg = wl.config(layout=layout, cull_mode=cull)
        masks = None if wl.isolated else vox.neighbour_masks(coords, full6=bool(cull))
        _, _, offs = oracle.gen_mesh_batch(cfg, coords, masks, wl.index_base)
        want = int(offs[-1])
        assert want > 0, name
        for threads in (1, 4):
            got = oracle.baseline_run(cfg, coords, masks, wl.index_base, threads)
            assert got == want, (name, threads, got, want)


def test_baseline_treats_neighbours_outside_the_batch_as_absent(vox, oracle):
    """A mask bit for a neighbour that is not in the batch finds no chunk in the lookup, so
    the border faces are emitted: the total equals the batch oracle's with that bit clear."""
    wl = vox.workload("heightmap")
    cfg = wl.config()
    coords = list(wl.coords[:64])
    claimed = [0x0F] * len(coords)
    inside = vox.neighbour_masks(coords)
    _, _, offs = oracle.gen_mesh_batch(cfg, coords, inside)
    assert oracle.baseline_run(cfg, coords, claimed, 0, 2) == int(offs[-1])
