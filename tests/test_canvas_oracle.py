"""The canvas oracle (oracle/vo_canvas.c) against the reference's own Canvas:
the committed fixture tests/golden/reference_canvas.npz (made from
src/voromesh/canvas.cpp by tests/golden/make_canvas_golden.py) and, where the
reference was compiled here (oracle/_ref), the live class on random edits.

States must agree up to a relabelling of slot indices: the reference hands
free slots to a stamp's rim voxels in std::unordered_map order
(canvas.cpp:200), the oracle in tile-major order. Everything else —
occupancy, surface masks and points, slot values, counts, free-list length,
the ordered list of removed slots — is identical."""
from pathlib import Path

import numpy as np
import pytest

import canvas_shapes

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_canvas.npz"


def _dense(z, prefix, tiles):
    spt = np.full((tiles * 64, 2), -1.0, np.float32)
    sslot = np.full(tiles * 64, -1, np.int32)
    vox = z[prefix + "vox"]
    spt[vox] = z[prefix + "pts"]
    sslot[vox] = z[prefix + "vslots"]
    return dict(inside=z[prefix + "inside"], smask=z[prefix + "smask"], spt=spt, sslot=sslot, slots=z[prefix + "slots"],
                free=z[prefix + "free"], counts=tuple(int(v) for v in z[prefix + "counts"]))


@pytest.mark.parametrize("name", ["heart96", "heart_odd"])
def test_oracle_matches_reference_fixture(orc, name):
    z = np.load(GOLDEN)
    w, h, vs = (float(v) for v in z[f"{name}/dims"])
    _, _, tx, ty = orc.canvas_dims(w, h, vs)
    c = orc.Canvas(w, h, vs)
    c.rasterize(z[f"{name}/poly"])
    pi = orc.canvas_relabelling(c.state(), _dense(z, f"{name}/s0/", tx * ty))
    # RasterizeShape allocates in tile-major order in both: no relabelling
    assert np.array_equal(pi, np.arange(len(pi)))
    edits, dirty = z[f"{name}/edits"], z[f"{name}/dirty"]
    off = 0
    checked = 0
    for k, (cx, cy, r, ins) in enumerate(z[f"{name}/stamps"]):
        e = c.stamp(cx, cy, r, int(ins))
        assert e.rect() + e.counts() == tuple(int(v) for v in edits[k][:7])
        n = int(edits[k][7])
        assert len(e.dirty) == n
        ref_dirty = dirty[off:off + n]
        off += n
        key = f"{name}/s{k + 1}/inside"
        if key in z.files:
            pi = orc.canvas_relabelling(c.state(), _dense(z, f"{name}/s{k + 1}/", tx * ty))
            assert sorted(pi[e.dirty[e.removed:]].tolist()) == sorted(ref_dirty[e.removed:].tolist())
            checked += 1
    assert checked >= 3


def test_oracle_matches_live_reference(orc):
    if not orc.ref_canvas_available():
        pytest.skip("the reference canvas is not compiled here")
    from voromesh_gb300 import synth

    for (w, vs, segs, seed) in [(1024.0, 1.0, 4096, 1), (100.0, 0.37, 50, 3), (64.0, 1.0, 7, 4)]:
        poly = synth.heart(0.5 * w, 0.5 * w, 0.8 * w, segs)
        a, b = orc.Canvas(w, w, vs), orc.RefCanvas(w, w, vs)
        a.rasterize(poly)
        b.rasterize(poly)
        pi = orc.canvas_relabelling(a.state(), b.state())
        assert np.array_equal(pi, np.arange(len(pi)))
        rng = np.random.default_rng(seed)
        for _ in range(30):
            cx, cy = rng.uniform(-0.1 * w, 1.1 * w, 2).astype(np.float32)
            r = np.float32(rng.uniform(0.5, 0.15 * w / vs) * vs)
            ins = bool(rng.integers(2))
            ea, eb = a.stamp(cx, cy, r, ins), b.stamp(cx, cy, r, ins)
            assert ea.rect() == eb.rect() and ea.counts() == eb.counts()
            # removed slots leave in the same (tile-major) order in both
            assert np.array_equal(pi[ea.dirty[:ea.removed]], eb.dirty[:eb.removed])
            pi = orc.canvas_relabelling(a.state(), b.state())
            assert sorted(pi[ea.dirty[ea.removed:]].tolist()) == sorted(eb.dirty[eb.removed:].tolist())


@pytest.mark.parametrize("name", canvas_shapes.NAMES)
def test_oracle_matches_live_reference_on_edge_shapes(orc, name):
    """Every shape the GPU parity tests use (self-intersecting, clockwise,
    600-crossing scanlines, mixed-magnitude coordinates in one voxel, a
    sliver, a single vertex), rasterised and then stamped, against the
    reference's own Canvas."""
    if not orc.ref_canvas_available():
        pytest.skip("the reference canvas is not compiled here")
    (w, h, vs), poly = canvas_shapes.shape(name)
    a, b = orc.Canvas(w, h, vs), orc.RefCanvas(w, h, vs)
    a.rasterize(poly)
    b.rasterize(poly)
    pi = orc.canvas_relabelling(a.state(), b.state())
    assert np.array_equal(pi, np.arange(len(pi)))
    rng = np.random.default_rng(sum(map(ord, name)))
    for _ in range(12):
        cx = np.float32(rng.uniform(-0.1 * w, 1.1 * w))
        cy = np.float32(rng.uniform(-0.1 * h, 1.1 * h))
        r = np.float32(rng.uniform(0.5, 0.2 * min(w, h) / vs) * vs)
        ins = bool(rng.integers(2))
        ea, eb = a.stamp(cx, cy, r, ins), b.stamp(cx, cy, r, ins)
        assert ea.rect() == eb.rect() and ea.counts() == eb.counts()
        assert np.array_equal(pi[ea.dirty[:ea.removed]], eb.dirty[:eb.removed])
        pi = orc.canvas_relabelling(a.state(), b.state())
        assert sorted(pi[ea.dirty[ea.removed:]].tolist()) == sorted(eb.dirty[eb.removed:].tolist())


def test_relabelling_check_catches_a_planted_error(orc):
    """The comparison itself: a changed point, occupancy bit or slot value in
    the oracle's state is reported."""
    from voromesh_gb300 import synth

    c = orc.Canvas(64.0, 64.0, 1.0)
    c.rasterize(synth.heart(32.0, 32.0, 50.0, 100))
    good = c.state()
    for key, mutate in [("inside", lambda a: a.__setitem__(3, a[3] ^ np.uint64(1))),
                        ("spt", lambda a: a.__setitem__(np.flatnonzero(a[:, 0] >= 0)[0], (1.0, 2.0))),
                        ("slots", lambda a: a.__setitem__(0, (7.0, 7.0)))]:
        bad = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in good.items()}
        mutate(bad[key])
        with pytest.raises(AssertionError):
            orc.canvas_relabelling(good, bad)
