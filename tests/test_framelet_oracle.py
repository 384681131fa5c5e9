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


# --------------------------------------------------------------------------
# Impulse responses written out by hand from the MATLAB sources
# --------------------------------------------------------------------------
# ConvSymAsym3D.m:19-24 places filter M at every 2^(L-1)-th tap of a column
# kernel and calls imfilter(A, ker, 'circular'): correlation (imfilter's
# default), 'same' size, kernel centre at its middle tap. For an impulse at
# index p that gives C(p - d * 2^(L-1)) = M(c + d) (c the middle tap): the
# filter read backwards around p, wrapped around the array's ends.
# FraDecMultiLevel3D.m:35-44: filter D{i} runs along MATLAB dimension 2 (y),
# D{j} along dimension 1 (x), D{k} along dimension 3 (z); here (z, y, x) is
# numpy's (axis 0, 1, 2). Linear filters, GenerateFrameletFilter.m:10-12:
#   D1 = [1 2 1]/4, D2 = -[1 0 -1]/4*sqrt(2) = [-s, 0, s] with s = sqrt(2)/4,
#   D3 = [-1 2 -1]/4.
S4 = np.sqrt(2.0) / 4
RESP = {  # offset d -> value, the filter read backwards (offset -1 holds the last tap)
    0: {-1: 0.25, 0: 0.5, 1: 0.25},
    1: {-1: S4, 0: 0.0, 1: -S4},
    2: {-1: -0.25, 0: 0.5, 1: -0.25},
}


def _impulse(shape, at):
    a = np.zeros(shape)
    a[at] = 1.0
    return a


@pytest.mark.parametrize("band", [(1, 0, 0), (0, 1, 2), (2, 2, 1), (1, 1, 1)])
def test_level1_impulse_response_is_the_reversed_tensor_filter(band):
    shape, at = (7, 8, 9), (3, 4, 5)
    c = N.frame_dec_level(_impulse(shape, at), N.filters("linear")[0], 1)[band]
    i, j, k = band                    # along y, x, z
    want = np.zeros(shape)
    for dz, vz in RESP[k].items():
        for dy, vy in RESP[i].items():
            for dx, vx in RESP[j].items():
                want[at[0] + dz, at[1] + dy, at[2] + dx] = vz * vy * vx
    assert np.allclose(c, want, atol=1e-15, rtol=0)


def test_level2_taps_are_two_apart():
    """ConvSymAsym3D.m:16-20: at level 2 the kernel is [M1 0 M2 0 M3]."""
    shape, at = (5, 11, 6), (2, 5, 3)
    c = N.frame_dec_level(_impulse(shape, at), N.filters("linear")[0], 2)[(1, 0, 0)]
    line = c[at[0], :, at[2]] / (0.5 * 0.5)        # D1 centre taps along x and z
    want = np.zeros(11)
    want[at[1] - 2], want[at[1] + 2] = S4, -S4
    assert np.allclose(line, want, atol=1e-15, rtol=0)


def test_circular_boundary_wraps_the_response():
    """imfilter(..., 'circular') (ConvSymAsym3D.m:24): an impulse at the first
    index reaches the last one."""
    shape = (4, 6, 5)
    c = N.frame_dec_level(_impulse(shape, (0, 0, 0)), N.filters("linear")[0], 1)[(0, 1, 0)]
    # D2 along x: offset -1 -> index nx-1 holds +s, offset +1 -> index 1 holds -s
    assert c[0, 0, 4] == pytest.approx(S4 * 0.5 * 0.5)
    assert c[0, 0, 1] == pytest.approx(-S4 * 0.5 * 0.5)
    assert c[3, 5, 4] == pytest.approx(S4 * 0.25 * 0.25)


def test_haar_filters_are_one_sided():
    """GenerateFrameletFilter.m:3-4: D1 = [0 1 1]/2, D2 = -[0 1 -1]/2: the
    response of an impulse at p sits at p and p - 1 only."""
    shape, at = (4, 4, 6), (1, 2, 3)
    c = N.frame_dec_level(_impulse(shape, at), N.filters("haar")[0], 1)[(0, 1, 0)]
    line = c[at[0], at[1], :] / (0.5 * 0.5)
    want = np.zeros(6)
    want[at[2]], want[at[2] - 1] = -0.5, 0.5        # D2 = [0, -1/2, 1/2] read backwards
    assert np.allclose(line, want, atol=1e-15, rtol=0)
