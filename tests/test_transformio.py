"""Transform files in the reference's text format (no GPU needed): the number
layout of NumberToString (shortest round trip, ECMAScript layout), the block
layout of the text writer, and read-back of affine, B-spline and composite
transforms."""
import numpy as np
import pytest

from itk_gb300 import AffineTransform, CompositeTransform, data
from itk_gb300.image import Image
from itk_gb300.transformio import ReadTransform, WriteTransform, number_to_string, transform_to_text, \
    transforms_from_text


@pytest.mark.parametrize("x,s", [
    (1.0, "1"), (0.0, "0"), (-0.0, "0"), (0.5, "0.5"), (0.1, "0.1"), (-2.25, "-2.25"), (100.0, "100"),
    (123.456, "123.456"), (1e-7, "1e-7"), (1.5e-7, "1.5e-7"), (1e-6, "0.000001"), (1.25e-6, "0.00000125"),
    (1e20, "100000000000000000000"), (1e21, "1e+21"), (1.5e22, "1.5e+22"), (5e-324, "5e-324"),
    (1.7976931348623157e308, "1.7976931348623157e+308"), (1 / 3, "0.3333333333333333"),
    (123456789012345680000.0, "123456789012345680000"), (0.000123, "0.000123"),
])
def test_number_to_string_layout(x, s):
    assert number_to_string(x) == s


def test_number_to_string_round_trips():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.normal(size=2000) * 10.0 ** rng.integers(-12, 12, size=2000),
                         rng.uniform(-1, 1, size=500)])
    for x in xs:
        assert float(number_to_string(x)) == x


def affine():
    t = AffineTransform()
    t.SetCenter([10.5, -3.0, 7.25])
    t.SetMatrix([[1.01, 0.02, -0.003], [0.0, 0.99, 0.1], [1e-7, 0.0, 1.0]])
    t.SetTranslation([0.5, -1.25, 3.0])
    return t


def test_affine_text_layout():
    t = AffineTransform()
    assert transform_to_text(t) == ("#Insight Transform File V1.0\n#Transform 0\n"
                                    "Transform: AffineTransform_double_3_3\n"
                                    "Parameters: 1 0 0 0 1 0 0 0 1 0 0 0\nFixedParameters: 0 0 0\n")


def test_round_trip_affine_bspline_composite(tmp_path):
    img = Image(np.zeros((20, 22, 24), np.float32), spacing=(1.0, 1.5, 0.8), origin=(1.0, 2.0, 3.0))
    b = data.random_bspline_coefficients(data.bspline_over_image(img, (4, 5, 3)), seed=3)
    a = affine()
    c = CompositeTransform()
    c.AddTransform(a)
    c.AddTransform(b)
    for t in (a, b, c):
        p = tmp_path / "t.tfm"
        WriteTransform(t, str(p))
        r = ReadTransform(str(p))
        assert type(r) is type(t)
        if isinstance(t, CompositeTransform):
            assert r.GetNumberOfTransforms() == 2
            for k in range(2):
                assert np.array_equal(r.GetNthTransform(k).GetParameters(), t.GetNthTransform(k).GetParameters())
                assert np.array_equal(r.GetNthTransform(k).GetFixedParameters(),
                                      t.GetNthTransform(k).GetFixedParameters())
        else:
            assert np.array_equal(r.GetParameters(), t.GetParameters())
            assert np.array_equal(r.GetFixedParameters(), t.GetFixedParameters())
        x = np.array([[3.0, 4.0, 5.0], [10.0, 12.0, 9.0]])
        assert np.array_equal(r.TransformPoint(x), t.TransformPoint(x))


def test_reader_accepts_parameters_before_fixed_parameters():
    text = ("#Insight Transform File V1.0\n#Transform 0\nTransform: BSplineTransform_double_3_3\n"
            "Parameters: " + " ".join(["0.5"] * (3 * 5 * 5 * 5)) + "\n"
            "FixedParameters: 5 5 5 -1 -1 -1 1 1 1 1 0 0 0 1 0 0 0 1\n")
    (t,) = transforms_from_text(text)
    assert t.GetNumberOfParameters() == 375 and np.all(t.GetParameters() == 0.5)


def test_reader_rejects_unknown_types_and_bad_tags():
    with pytest.raises(ValueError):
        transforms_from_text("#Insight Transform File V1.0\nTransform: AffineTransform_double_10_10\n")
    with pytest.raises(ValueError):
        transforms_from_text("Transform AffineTransform_double_3_3\n")


def test_round_trip_displacement_field_and_composite(tmp_path):
    from itk_gb300 import DisplacementFieldImage, DisplacementFieldTransform
    img = Image(np.zeros((5, 6, 7), np.float32), spacing=(1.0, 1.5, 0.8), origin=(1.0, 2.0, 3.0))
    F = DisplacementFieldTransform()
    F.SetDisplacementField(DisplacementFieldImage.like(img, np.random.default_rng(2).normal(size=(5, 6, 7, 3))))
    C = CompositeTransform()
    C.AddTransform(affine())
    C.AddTransform(F)
    for t in (F, C):
        p = tmp_path / "f.tfm"
        WriteTransform(t, str(p))
        r = ReadTransform(str(p))
        assert type(r) is type(t)
        assert np.array_equal(r.GetParameters(), t.GetParameters())
        assert np.array_equal(r.GetFixedParameters(), t.GetFixedParameters())
        x = np.array([[3.0, 4.0, 5.0], [6.0, 9.0, 4.0]])
        assert np.array_equal(r.TransformPoint(x), t.TransformPoint(x))
