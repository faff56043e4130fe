"""GB300-native ITK registration-metric hot path.

GetValueAndDerivative of MeanSquaresImageToImageMetricv4 and
MattesMutualInformationImageToImageMetricv4 on Image<float,3> under affine,
B-spline, [affine, B-spline] composite and displacement-field transforms (and
CorrelationImageToImageMetricv4 and JointHistogramMutualInformationImageToImageMetricv4
under affine and B-spline transforms), computed by hand-written
sm_103a CUDA kernels behind the C ABI in include/itk_gb300.h.
"""
from ._capi import ExceptionObject, lib, library_path
from .batch import RegistrationBatch
from .filters import (GradientRecursiveGaussianImageFilter, ShrinkImageFilter, SmoothingRecursiveGaussianImageFilter,
                      shrink_geometry)
from .image import DisplacementFieldImage, GradientImage, Image
from .metrics import (CorrelationImageToImageMetricv4, ImageToImageMetricv4,
                      JointHistogramMutualInformationImageToImageMetricv4,
                      MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4, context)
from .optimizers import RegularStepGradientDescentOptimizerv4
from .registration import ImageRegistrationMethodv4, sample_count, sample_points
from .scales import RegistrationParameterScalesFromPhysicalShift
from .serving import RegistrationRequest, RegistrationResult, RegistrationServer
from .transformio import ReadTransform, WriteTransform
from .transforms import AffineTransform, BSplineTransform, CompositeTransform, DisplacementFieldTransform

__all__ = [
    "AffineTransform", "BSplineTransform", "CompositeTransform", "CorrelationImageToImageMetricv4", "ExceptionObject",
    "DisplacementFieldImage", "DisplacementFieldTransform", "GradientImage",
    "GradientRecursiveGaussianImageFilter", "Image", "ImageRegistrationMethodv4", "ImageToImageMetricv4",
    "JointHistogramMutualInformationImageToImageMetricv4",
    "MattesMutualInformationImageToImageMetricv4", "MeanSquaresImageToImageMetricv4",
    "RegistrationBatch", "RegistrationParameterScalesFromPhysicalShift", "RegistrationRequest", "RegistrationResult",
    "RegistrationServer",
    "RegularStepGradientDescentOptimizerv4", "ShrinkImageFilter", "SmoothingRecursiveGaussianImageFilter", "context",
    "ReadTransform", "WriteTransform", "lib", "library_path", "sample_count", "sample_points", "shrink_geometry",
]
