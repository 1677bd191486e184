"""Synthetic cube generator: layout, determinism, scatterer placement.  CPU only."""
import numpy as np

from cos_gb300 import synth


def test_layout_and_determinism():
    a = synth.cube(64, 8, 16, [10.0], seed=3)
    b = synth.cube(64, 8, 16, [10.0], seed=3)
    assert a.shape == (8, 64, 16) and a.dtype == np.complex64 and a.flags.c_contiguous
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, synth.cube(64, 8, 16, [10.0], seed=4))


def test_noise_power_and_scatterer():
    x = synth.cube(256, 16, 32, [], seed=1)
    assert abs(np.mean(np.abs(x) ** 2) - 1.0) < 0.02
    y = synth.cube(256, 16, 32, [100.0], seed=1)
    d = y - x
    # on its own beam the phase ramp is flat: the channel sum is coherent there
    b0 = int(np.argmax(np.abs(d.sum(axis=2)).sum(axis=1)))
    row = np.argmax(np.abs(d[b0, :, 0]))
    np.testing.assert_allclose(d[b0, row], d[b0, row, 0], rtol=1e-5)
    assert abs(abs(d[b0, row, 0]) - 100.0) < 5.0


def test_coherent_pair():
    x = synth.cube(64, 8, 16, [100.0, 100.0], 3, coherent_pair=True)
    n = synth.cube(64, 8, 16, [], 3)
    d = np.abs((x - n).sum(axis=2)).sum(axis=1)
    beams = np.nonzero(d > 0.5 * d.max())[0]
    assert len(beams) >= 2 and beams[1] - beams[0] == 1
