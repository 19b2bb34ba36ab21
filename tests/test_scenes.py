"""Scene generators: the batched-scene packer keeps scenes apart (CPU)."""
import numpy as np

from mpm_gb300 import scenes


def _batch():
    sc = scenes.batch_scenes(n_scenes=10, n_min=200, n_max=6000, sizes=(12, 16, 20), seed=77)
    return scenes.pack_scenes(sc)


def test_packing_keeps_scenes_apart():
    b = _batch()
    nn = b.scene.xynodec
    owner = -np.ones(b.scene.nodec, dtype=np.int64)
    for i, s in enumerate(b.scenes):
        o = b.cell_offset[i]
        gx, gy, gz = s.xyelem
        ii, jj, kk = np.meshgrid(np.arange(gx + 1) + o[0], np.arange(gy + 1) + o[1], np.arange(gz + 1) + o[2],
                                 indexing="ij")
        ids = (ii + nn[0] * (jj + nn[1] * kk)).ravel()
        assert np.all(owner[ids] == -1)
        owner[ids] = i


def test_packing_preserves_particles_and_materials():
    b = _batch()
    assert b.scene.num == sum(s.num for s in b.scenes)
    for i, s in enumerate(b.scenes):
        sl = slice(b.begin[i], b.end[i])
        assert np.allclose(b.local(i, b.scene.coord[sl]), s.coord, rtol=0, atol=1e-12)
        assert np.all(b.scene.matid[sl] == i)
        assert np.array_equal(b.scene.mat_prop[i], s.mat_prop[0])


def test_full_batch_size():
    sc = scenes.batch_scenes()
    assert len(sc) == 256
    n = np.array([s.num for s in sc])
    assert 3.0e6 < n.sum() < 8.0e6 and n.min() >= 500 and n.max() <= 2.0e5
