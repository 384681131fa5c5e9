"""The reference's analytic known answers (testBall.m) through the oracle:
unit-disc fan chords and the cone-beam unit ball (circle and helix, including
the normalised output yNorm). Errors are the pixelisation of the phantom."""
import oracle as O
from tests.known_answers import cone_ball, fan_disc, fan_disc_beam, rel


def test_fan_unit_disc_chords():
    p, x, ex = fan_disc()
    assert rel(O.fan_siddon_f32(x, p), ex) < 5e-3
    assert rel(O.fan_gao_f32(x, p), ex) < 5e-3
    assert rel(O.exact_forward(x, p), ex) < 5e-3


def test_fan_unit_disc_finite_beam():
    p, x, ex = fan_disc_beam()
    assert rel(O.fan_fb_f32(x, p, threads=8), ex) < 5e-3


def test_cone_unit_ball_circle():
    p, x, ex, exn = cone_ball(scan="circle")
    assert rel(O.cone_siddon_f32(x, p, threads=8), ex) < 3e-2
    y, yn = O.cone_gao_f32(x, p, threads=8)
    assert rel(y, ex) < 3e-2 and rel(yn, exn) < 3e-2


def test_cone_unit_ball_helix_with_ynorm():
    p, x, ex, exn = cone_ball(scan="helix")
    y, yn = O.cone_gao_f32(x, p, threads=8)
    assert rel(y, ex) < 3e-2
    assert rel(yn, exn) < 3e-2
