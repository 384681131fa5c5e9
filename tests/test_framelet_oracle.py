"""CPU pins of the FP64 framelet restatement (oracle/numerics.py), which the
GPU framelet tests use as their checker. MATLAB is not available, so the
restatement is pinned by the reference's own known answer -- perfect
reconstruction, W^T W = I (testFramelet.m:31) -- and by properties the
filter banks of GenerateFrameletFilter.m:2-30 imply: the decomposition is a
tight frame (it keeps the energy) and linear, and softThreshold.m:65-78
leaves each level's low-pass band alone."""
import numpy as np
import pytest

from oracle import numerics as N

KINDS = ["linear", "haar", "cubic"]


def _vol(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("levels", [1, 2, 3])
def test_perfect_reconstruction(kind, levels):
    u = _vol((8, 12, 16), seed=levels)
    rec = N.frame_rec(N.frame_dec(u, levels=levels, kind=kind), kind=kind)
    assert np.max(np.abs(rec - u)) < 1e-12 * np.max(np.abs(u))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("levels", [1, 2])
def test_decomposition_keeps_the_energy(kind, levels):
    """Tight frame: the energy of every band that is not decomposed further
    (all bands of the last level, the high-pass bands of the others) adds up
    to the energy of the volume."""
    u = _vol((8, 8, 8), seed=7)
    c = N.frame_dec(u, levels=levels, kind=kind)
    e = 0.0
    for lev, bands in enumerate(c):
        for key, a in bands.items():
            if key == (0, 0, 0) and lev < levels - 1:
                continue
            e += float(np.sum(a * a))
    assert abs(e - float(np.sum(u * u))) < 1e-10 * float(np.sum(u * u))


def test_band_count_and_shapes():
    for kind, nf in (("linear", 3), ("haar", 2), ("cubic", 5)):
        c = N.frame_dec(_vol((4, 6, 8), seed=1), levels=2, kind=kind)
        assert len(c) == 2
        for bands in c:
            assert len(bands) == nf ** 3
            assert all(a.shape == (4, 6, 8) for a in bands.values())


@pytest.mark.parametrize("kind", KINDS)
def test_decomposition_is_linear(kind):
    a, b = _vol((6, 6, 6), seed=2), _vol((6, 6, 6), seed=3)
    ca, cb = N.frame_dec(a, 2, kind), N.frame_dec(b, 2, kind)
    cab = N.frame_dec(2.0 * a - 0.5 * b, 2, kind)
    for la, lb, lab in zip(ca, cb, cab):
        for key in lab:
            assert np.allclose(lab[key], 2.0 * la[key] - 0.5 * lb[key], atol=1e-12)


def test_constant_volume_lives_in_the_low_pass():
    """The low-pass filters sum to 1 and the others to 0: a constant volume
    has only low-pass coefficients, equal to the constant."""
    u = np.full((6, 8, 10), 3.25)
    for kind in KINDS:
        c = N.frame_dec(u, 2, kind)
        for bands in c:
            for key, a in bands.items():
                want = 3.25 if key == (0, 0, 0) else 0.0
                assert np.allclose(a, want, atol=1e-12), (kind, key)


def test_soft_shrink_known_answers():
    a = np.array([-2.0, -0.5, 0.0, 0.5, 2.0]).reshape(1, 1, 5)
    coefs = [{(0, 0, 0): a.copy(), (1, 0, 0): a.copy(), (0, 2, 1): a.copy()}]
    out = N.shrink(coefs, 1.0)
    assert np.array_equal(out[0][(0, 0, 0)], a)                       # low-pass kept
    for key in ((1, 0, 0), (0, 2, 1)):
        assert np.array_equal(out[0][key].ravel(), [-1.0, 0.0, 0.0, 0.0, 1.0])
