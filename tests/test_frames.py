"""
Device frame files (CPU): ``batch.save_frames`` streams frames into the
file format of ``myokit.DataBlock2d.save`` / ``DataBlock1d.save``
(``myokit/_datablock.py:1423-1500, 631-704``). The archive's header and
data are byte-identical to what the reference writes for the same block,
and the reference's loaders read it back exactly.
"""
import os
import zipfile

import numpy as np
import pytest
import torch

from conftest import myokit
from myokit_gb300.batch import frames_to_block, save_frames


def _frames(shape, seed=0):
    rng = np.random.default_rng(seed)
    return torch.tensor(rng.normal(size=shape), dtype=torch.float32)


@pytest.mark.parametrize('chunk', [1, 3, 100])
def test_same_bytes_as_reference_block_2d(tmp_path, chunk):
    fr = _frames((7, 5, 6))
    t = np.arange(7) * 5.0
    a, b = str(tmp_path / 'a.zip'), str(tmp_path / 'b.zip')
    save_frames(a, t, fr, chunk=chunk)
    frames_to_block(t, fr).save(b)
    za, zb = zipfile.ZipFile(a), zipfile.ZipFile(b)
    for entry in ('header_block2d.txt', 'data.bin'):
        assert za.read(entry) == zb.read(entry)
    blk = myokit.DataBlock2d.load(a)
    assert blk.shape() == (7, 5, 6)
    assert np.array_equal(blk.time(), t)
    assert np.array_equal(blk.get2d('membrane.V'), fr.double().numpy())


def test_several_variables_and_1d(tmp_path):
    t = np.linspace(0, 10, 4)
    sets = {'membrane.V': _frames((4, 3, 8), 1),
            'ica.Ca_i': np.abs(_frames((4, 3, 8), 2).numpy())}
    p = str(tmp_path / 'two.zip')
    save_frames(p, t, sets, chunk=3)
    blk = myokit.DataBlock2d.load(p)
    assert set(blk.keys2d()) == set(sets)
    for k, v in sets.items():
        assert np.array_equal(blk.get2d(k), np.asarray(v, dtype=float))
    # 1D frames (n, nx) give a DataBlock1d file
    f1 = _frames((5, 9), 3)
    p1 = str(tmp_path / 'one.zip')
    save_frames(p1, np.arange(5.0), f1, name='membrane.V', chunk=2)
    b1 = myokit.DataBlock1d.load(p1)
    assert np.array_equal(b1.get1d('membrane.V'), f1.double().numpy())
    ref = myokit.DataBlock1d(9, np.arange(5.0))
    ref.set1d('membrane.V', f1.double().numpy())
    ref.save(str(tmp_path / 'ref1.zip'))
    assert (zipfile.ZipFile(p1).read('data.bin') ==
            zipfile.ZipFile(str(tmp_path / 'ref1.zip')).read('data.bin'))


def test_argument_checks(tmp_path):
    p = str(tmp_path / 'x.zip')
    with pytest.raises(ValueError, match='one time per frame'.capitalize()):
        save_frames(p, np.arange(3.0), _frames((4, 2, 2)))
    with pytest.raises(ValueError, match='same shape'):
        save_frames(p, np.arange(2.0), {'a': _frames((2, 2, 2)),
                                        'b': _frames((2, 3, 2))})
    with pytest.raises(ValueError, match='shaped'):
        save_frames(p, np.arange(2.0), _frames((2, 2, 2, 2)))
    with pytest.raises(ValueError, match='No frames'):
        save_frames(p, np.arange(2.0), {})
    assert not os.path.exists(p)
