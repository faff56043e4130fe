"""Writes tests/golden/reference_known_values.json.

The numbers come from the reference's own unit tests (read as text, cited
below) and from closed forms of the reference's test inputs; nothing here runs
the reference.  Run: python tests/golden/make_golden.py
"""
import json
import os
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def mean_squares_closed_form():
    """Registration/Metricsv4/test/itkMeanSquaresImageToImageMetricv4Test.cxx:33-72: 5^3 images,
    fixed voxel n = count^2, moving voxel = 1/count^2 (count = 1..125, x fastest), identity
    transforms, dense.  For Image<float,3> the pixel values and the difference are float
    (FixedImagePixelType), so value = mean(float(float(n^2) - float(1/n^2))^2)."""
    total = Fraction(0)
    total_double = Fraction(0)
    for c in range(1, 126):
        f = np.float32(c * c)
        m = np.float32(1.0 / (c * c))
        d = np.float32(f - m)
        total += Fraction(float(d)) ** 2
        total_double += (Fraction(c * c) - Fraction(1, c * c)) ** 2
    return float(total / 125), float(total_double / 125)


def main():
    msq_float, msq_double = mean_squares_closed_form()
    out = {
        "mattes_2d_known_values": {
            "source": "Registration/Metricsv4/test/itkMattesMutualInformationImageToImageMetricv4Test.cxx:386-401",
            "setup": "100x100 Image<double,2>, spacing (3,2), origin (0.001,-0.002), fixed = uchar(200 exp(-r^2/s^2)) "
                     "centred at (50,50), s = 50; moving the same shifted by (5,5) index; AffineTransform identity "
                     "(centre 0); 50 bins; central-difference gradients; dense, or every 5th fixed voxel as a fixed "
                     "sampled point set",
            "values": [-1.297994750907097, -1.297995377157083, -1.297994448222851, -1.297995700722833],
            "order": "GetValue at parameters[k] + delta, - delta, + 2 delta, - 2 delta; delta = 1e-5",
            "value_tolerance": 0.05,
            "fd_ratio_tolerance_dense": 0.014,
            "fd_ratio_tolerance_sampled": 0.075,
            "get_value_vs_get_value_and_derivative_ulps": 8,
        },
        "mean_squares_5cube": {
            "source": "Registration/Metricsv4/test/itkMeanSquaresImageToImageMetricv4Test.cxx:33-72",
            "value_float_pixels": msq_float,
            "value_double_pixels": msq_double,
            "nvalid": 125,
        },
        "linear_interpolation": {
            "source": "Core/ImageFunction/test/itkLinearInterpolateImageFunctionTest.cxx:100-205",
            "setup": "voxel value 3*x + y + z; inside-buffer points are interpolated exactly",
            "tolerance": 5e-6,
        },
        "bspline_kernel": {
            "source": "Core/Common/include/itkBSplineKernelFunction.h:152-169",
            "values": {"0": 2.0 / 3.0, "0.5": 23.0 / 48.0, "1": 1.0 / 6.0, "1.5": 1.0 / 48.0, "2": 0.0},
            "derivative": {"0.5": -0.625, "-0.5": 0.625, "1.5": -0.125, "0": 0.0},
        },
    }
    with open(os.path.join(HERE, "reference_known_values.json"), "w") as f:
        json.dump(out, f, indent=2, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
