"""ctypes front end of the FP64 CPU oracle (oracle/itk_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the GPU library:
tests, ``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` use it.  Nothing in ``itk_gb300`` imports this module.

Arrays follow ITK's memory order: a 3-D image is a numpy array of shape
(nz, ny, nx), x fastest; a gradient image is (nz, ny, nx, 3) float64 like
``Image<CovariantVector<double,3>,3>``; sample points are (n, 3) float32 like
``PointSet<float,3>`` (Registration/RegistrationMethodsv4/include/
itkImageRegistrationMethodv4.hxx:925-1003 stores them as float).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libitk_oracle.so")
_lib = None

TRANSFORM_AFFINE = 0
TRANSFORM_BSPLINE = 1
TRANSFORM_COMPOSITE = 2
TRANSFORM_DISPLACEMENT = 3

STATUS_NAMES = {
    0: "OK",
    1: "BAD_ARG",
    2: "NO_VALID_POINTS",
    3: "JOINT_PDF_SUM_ZERO",
    4: "FIXED_CONSTANT",
    5: "MOVING_CONSTANT",
    6: "FIXED_EMPTY",
    7: "MOVING_EMPTY",
    8: "OOM",
}


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (portable C, no ISA flags)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                          for f in ("itk_oracle.c", "itk_oracle_filters.c", "itk_oracle_sampling.c",
                                                    "itk_oracle.h"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_msq_flat.argtypes = [P, P, P, P, P, P, P, P, i64, ctypes.c_int, P, i64, P, i64,
                                   ctypes.c_int, ctypes.c_int, P, P, P]
        L.orc_mattes_flat.argtypes = [P, P, P, P, P, P, P, P, i64, ctypes.c_int, P, i64, P, i64,
                                      i64, ctypes.c_int, ctypes.c_int, P, P, P, P, P]
        L.orc_msq_flat_v.argtypes = L.orc_msq_flat.argtypes + [P, P]
        L.orc_corr_flat_v.argtypes = L.orc_msq_flat_v.argtypes
        L.orc_msq_flat_fpc.argtypes = L.orc_msq_flat.argtypes + [ctypes.c_double]
        L.orc_mattes_flat_v.argtypes = L.orc_mattes_flat.argtypes + [P, P]
        L.orc_jhmi_flat_v.argtypes = [P, P, P, P, P, P, P, P, i64, ctypes.c_int, P, i64, P, i64, i64,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]
        L.orc_gaussian_kernel.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, P, ctypes.c_int]
        L.orc_transform_point_flat.argtypes = [ctypes.c_int, P, i64, P, i64, P, i64, P]
        L.orc_interpolate_flat.argtypes = [P, P, P, P, i64, P, P]
        L.orc_central_difference_flat.argtypes = [P, P, P, P, i64, P]
        L.orc_bspline_weights.argtypes = [P, P, P]
        L.orc_bspline3.argtypes = [ctypes.c_double]
        L.orc_bspline3.restype = ctypes.c_double
        L.orc_bspline3_derivative.argtypes = [ctypes.c_double]
        L.orc_bspline3_derivative.restype = ctypes.c_double
        d, ci = ctypes.c_double, ctypes.c_int
        L.orc_rg_setup.argtypes = [d, d, ci, ci, P]
        L.orc_rg_filter_line.argtypes = [P, P, P, P, i64]
        L.orc_smooth_recursive_gaussian.argtypes = [P, P, P, P, P]
        L.orc_gradient_recursive_gaussian.argtypes = [P, P, P, P, P, d, ci, ci]
        L.orc_shrink_geometry.argtypes = [P] * 8
        u32 = ctypes.c_uint32
        L.orc_mt_sequence.argtypes = [u32, i64, P, i64]
        L.orc_mt_normals.argtypes = [u32, P, i64]
        L.orc_sample_points.argtypes = [ci, P, P, d, ctypes.c_int32, P, i64, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Geometry:
    """Image geometry as ITK's ImageBase holds it (start index 0)."""
    size: tuple          # (nx, ny, nz)
    spacing: tuple = (1.0, 1.0, 1.0)
    origin: tuple = (0.0, 0.0, 0.0)
    direction: tuple = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)

    def flat(self):
        return np.ascontiguousarray(np.array(list(self.spacing) + list(self.origin) + list(self.direction),
                                             dtype=np.float64))

    def size_array(self):
        return np.ascontiguousarray(np.array(self.size, dtype=np.int64))


@dataclass
class Transform:
    """Flat transform description (see itk_oracle.h for the encodings)."""
    kind: int
    params: np.ndarray
    fixed: np.ndarray

    @property
    def nparams(self):
        return int(self.params.size)


def _img(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _grad(g):
    return None if g is None else np.ascontiguousarray(g, dtype=np.float64)


def _pts(p):
    return None if p is None else np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(-1, 3))


def _vgeom(g):
    return (None, None) if g is None else (g.size_array(), g.flat())


def _threads(nthreads, pixel_double):
    t = int(nthreads or os.cpu_count()) & 0xFFFF
    return t | (0x10000 if pixel_double else 0)


def mean_squares(fixed, fgeom, moving, mgeom, transform, moving_grad=None, points=None, nthreads=None,
                 compute_derivative=True, pixel_double=False, virtual_geom=None):
    """Returns (status, value, derivative, nvalid).  virtual_geom: the dense virtual
    domain (default: the fixed image's geometry)."""
    L = lib()
    fixed, moving = _img(fixed), _img(moving)
    mg, pts = _grad(moving_grad), _pts(points)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    value = np.zeros(1, np.float64)
    deriv = np.zeros(tp.size, np.float64)
    nvalid = np.zeros(1, np.uint64)
    fs, fg, ms, mgeo = fgeom.size_array(), fgeom.flat(), mgeom.size_array(), mgeom.flat()
    vs, vg = _vgeom(virtual_geom)
    rc = L.orc_msq_flat_v(_p(fixed), _p(fs), _p(fg), _p(moving), _p(ms), _p(mgeo), _p(mg), _p(pts),
                          0 if pts is None else pts.shape[0], transform.kind, _p(tp), tp.size, _p(tf), tf.size,
                          _threads(nthreads, pixel_double), int(compute_derivative), _p(value), _p(deriv),
                          _p(nvalid), _p(vs), _p(vg))
    return rc, float(value[0]), deriv, int(nvalid[0])


def mean_squares_fpc(fixed, fgeom, moving, mgeom, transform, resolution, moving_grad=None, points=None, nthreads=None):
    """MeanSquares with UseFloatingPointCorrection at `resolution`.  Returns (status, value, derivative, nvalid)."""
    L = lib()
    fixed, moving = _img(fixed), _img(moving)
    mg, pts = _grad(moving_grad), _pts(points)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    value = np.zeros(1, np.float64)
    deriv = np.zeros(tp.size, np.float64)
    nvalid = np.zeros(1, np.uint64)
    fs, fg, ms, mgeo = fgeom.size_array(), fgeom.flat(), mgeom.size_array(), mgeom.flat()
    rc = L.orc_msq_flat_fpc(_p(fixed), _p(fs), _p(fg), _p(moving), _p(ms), _p(mgeo), _p(mg), _p(pts),
                            0 if pts is None else pts.shape[0], transform.kind, _p(tp), tp.size, _p(tf), tf.size,
                            _threads(nthreads, False), 1, _p(value), _p(deriv), _p(nvalid), float(resolution))
    return rc, float(value[0]), deriv, int(nvalid[0])


def correlation(fixed, fgeom, moving, mgeom, transform, moving_grad=None, points=None, nthreads=None,
                compute_derivative=True, pixel_double=False, virtual_geom=None):
    """CorrelationImageToImageMetricv4.  Returns (status, value, derivative, nvalid)."""
    L = lib()
    fixed, moving = _img(fixed), _img(moving)
    mg, pts = _grad(moving_grad), _pts(points)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    value = np.zeros(1, np.float64)
    deriv = np.zeros(tp.size, np.float64)
    nvalid = np.zeros(1, np.uint64)
    fs, fg, ms, mgeo = fgeom.size_array(), fgeom.flat(), mgeom.size_array(), mgeom.flat()
    vs, vg = _vgeom(virtual_geom)
    rc = L.orc_corr_flat_v(_p(fixed), _p(fs), _p(fg), _p(moving), _p(ms), _p(mgeo), _p(mg), _p(pts),
                           0 if pts is None else pts.shape[0], transform.kind, _p(tp), tp.size, _p(tf), tf.size,
                           _threads(nthreads, pixel_double), int(compute_derivative), _p(value), _p(deriv),
                           _p(nvalid), _p(vs), _p(vg))
    return rc, float(value[0]), deriv, int(nvalid[0])


def joint_histogram_mi(fixed, fgeom, moving, mgeom, transform, bins=20, variance=1.5, moving_grad=None, points=None,
                       nthreads=None, compute_derivative=True, pixel_double=False, virtual_geom=None):
    """JointHistogramMutualInformationImageToImageMetricv4.  Returns (status, value,
    derivative, nvalid, smoothed joint PDF [moving bin, fixed bin])."""
    L = lib()
    fixed, moving = _img(fixed), _img(moving)
    mg, pts = _grad(moving_grad), _pts(points)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    value = np.zeros(1, np.float64)
    deriv = np.zeros(tp.size, np.float64)
    nvalid = np.zeros(1, np.uint64)
    pdf = np.zeros((bins, bins), np.float64)
    fs, fg, ms, mgeo = fgeom.size_array(), fgeom.flat(), mgeom.size_array(), mgeom.flat()
    vs, vg = _vgeom(virtual_geom)
    rc = L.orc_jhmi_flat_v(_p(fixed), _p(fs), _p(fg), _p(moving), _p(ms), _p(mgeo), _p(mg), _p(pts),
                           0 if pts is None else pts.shape[0], transform.kind, _p(tp), tp.size, _p(tf), tf.size,
                           int(bins), float(variance), _threads(nthreads, pixel_double), int(compute_derivative),
                           _p(value), _p(deriv), _p(nvalid), _p(pdf), _p(vs), _p(vg))
    return rc, float(value[0]), deriv, int(nvalid[0]), pdf


def gaussian_kernel(variance, max_error=0.01, max_width=32):
    """GaussianOperator coefficients (2 r + 1 values)."""
    c = np.zeros(129, np.float64)
    r = lib().orc_gaussian_kernel(float(variance), float(max_error), int(max_width), _p(c), 129)
    if r < 0:
        raise ValueError("kernel too wide")
    return c[:2 * r + 1].copy()


def mattes(fixed, fgeom, moving, mgeom, transform, bins=50, moving_grad=None, points=None, nthreads=None,
           compute_derivative=True, pixel_double=False, virtual_geom=None):
    """Returns (status, value, derivative, nvalid, joint_pdf[bins,bins], state[8])."""
    L = lib()
    fixed, moving = _img(fixed), _img(moving)
    mg, pts = _grad(moving_grad), _pts(points)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    b = max(int(bins), 5)
    value = np.zeros(1, np.float64)
    deriv = np.zeros(tp.size, np.float64)
    nvalid = np.zeros(1, np.uint64)
    pdf = np.zeros((b, b), np.float64)
    state = np.zeros(8, np.float64)
    fs, fg, ms, mgeo = fgeom.size_array(), fgeom.flat(), mgeom.size_array(), mgeom.flat()
    vs, vg = _vgeom(virtual_geom)
    rc = L.orc_mattes_flat_v(_p(fixed), _p(fs), _p(fg), _p(moving), _p(ms), _p(mgeo), _p(mg), _p(pts),
                             0 if pts is None else pts.shape[0], transform.kind, _p(tp), tp.size, _p(tf), tf.size,
                             b, _threads(nthreads, pixel_double), int(compute_derivative), _p(value), _p(deriv),
                             _p(nvalid), _p(pdf), _p(state), _p(vs), _p(vg))
    return rc, float(value[0]), deriv, int(nvalid[0]), pdf, state


def transform_points(transform, x):
    L = lib()
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 3))
    y = np.zeros_like(x)
    tp = np.ascontiguousarray(transform.params, dtype=np.float64)
    tf = np.ascontiguousarray(transform.fixed, dtype=np.float64)
    rc = L.orc_transform_point_flat(transform.kind, _p(tp), tp.size, _p(tf), tf.size, _p(x), x.shape[0], _p(y))
    if rc:
        raise ValueError(f"oracle transform error {STATUS_NAMES.get(rc, rc)}")
    return y


def interpolate(img, geom, points):
    L = lib()
    img = _img(img)
    pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
    vals = np.zeros(pts.shape[0], np.float64)
    inside = np.zeros(pts.shape[0], np.int32)
    rc = L.orc_interpolate_flat(_p(img), _p(geom.size_array()), _p(geom.flat()), _p(pts), pts.shape[0],
                                _p(vals), _p(inside))
    if rc:
        raise ValueError(f"oracle interpolate error {STATUS_NAMES.get(rc, rc)}")
    return vals, inside.astype(bool)


def central_difference(img, geom, points):
    L = lib()
    img = _img(img)
    pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
    g = np.zeros_like(pts)
    rc = L.orc_central_difference_flat(_p(img), _p(geom.size_array()), _p(geom.flat()), _p(pts),
                                       pts.shape[0], _p(g))
    if rc:
        raise ValueError(f"oracle central difference error {STATUS_NAMES.get(rc, rc)}")
    return g


def bspline_weights(cindex):
    L = lib()
    ci = np.ascontiguousarray(np.asarray(cindex, np.float64).reshape(3))
    w = np.zeros(64, np.float64)
    st = np.zeros(3, np.int64)
    L.orc_bspline_weights(_p(ci), _p(w), _p(st))
    return w, st


class RGCoef(ctypes.Structure):
    """orc_rg_coef: RecursiveGaussianImageFilter's IIR coefficients."""
    _fields_ = [(n, ctypes.c_double) for n in
                ("N0", "N1", "N2", "N3", "D1", "D2", "D3", "D4", "M1", "M2", "M3", "M4",
                 "BN1", "BN2", "BN3", "BN4", "BM1", "BM2", "BM3", "BM4")]


def rg_coefficients(sigma, spacing=1.0, order=0, normalize_across_scale=False):
    c = RGCoef()
    rc = lib().orc_rg_setup(float(sigma), float(spacing), int(order), int(normalize_across_scale),
                            ctypes.addressof(c))
    if rc:
        raise ValueError(f"oracle rg_setup error {STATUS_NAMES.get(rc, rc)}")
    return c


def rg_filter_line(line, sigma, spacing=1.0, order=0, normalize_across_scale=False):
    """RecursiveGaussianImageFilter on one 1-D line (FilterDataArray in double)."""
    c = rg_coefficients(sigma, spacing, order, normalize_across_scale)
    data = np.ascontiguousarray(np.asarray(line, np.float64))
    outs = np.zeros_like(data)
    scratch = np.zeros_like(data)
    lib().orc_rg_filter_line(ctypes.addressof(c), _p(data), _p(outs), _p(scratch), data.size)
    return outs


def smooth_recursive_gaussian(img, spacing, sigma):
    """SmoothingRecursiveGaussianImageFilter<Image<float,3>> (sigma per axis, physical units)."""
    a = _img(img)
    out = np.zeros_like(a)
    size = np.array([a.shape[2], a.shape[1], a.shape[0]], np.int64)
    sp = np.asarray(spacing, np.float64).reshape(3)
    sg = np.broadcast_to(np.asarray(sigma, np.float64), (3,)).copy()
    rc = lib().orc_smooth_recursive_gaussian(_p(a), _p(out), _p(size), _p(sp), _p(sg))
    if rc:
        raise ValueError(f"oracle smoothing error {STATUS_NAMES.get(rc, rc)}")
    return out


def gradient_recursive_gaussian(img, spacing, direction, sigma, normalize_across_scale=True,
                                use_image_direction=True):
    """GradientRecursiveGaussianImageFilter<Image<float,3>>: (nz, ny, nx, 3) float64."""
    a = _img(img)
    out = np.zeros(a.shape + (3,), np.float64)
    size = np.array([a.shape[2], a.shape[1], a.shape[0]], np.int64)
    sp = np.asarray(spacing, np.float64).reshape(3)
    d = np.ascontiguousarray(np.asarray(direction, np.float64).reshape(9))
    rc = lib().orc_gradient_recursive_gaussian(_p(a), _p(out), _p(size), _p(sp), _p(d), ctypes.c_double(sigma),
                                               int(normalize_across_scale), int(use_image_direction))
    if rc:
        raise ValueError(f"oracle gradient error {STATUS_NAMES.get(rc, rc)}")
    return out


def shrink_geometry(size_xyz, spacing, origin, direction, factors):
    """ShrinkImageFilter output (size, spacing, origin)."""
    sz = np.asarray(size_xyz, np.int64).reshape(3)
    sp = np.asarray(spacing, np.float64).reshape(3)
    org = np.asarray(origin, np.float64).reshape(3)
    d = np.ascontiguousarray(np.asarray(direction, np.float64).reshape(9))
    f = np.asarray(factors, np.int64).reshape(3)
    osz = np.zeros(3, np.int64)
    osp = np.zeros(3, np.float64)
    oorg = np.zeros(3, np.float64)
    lib().orc_shrink_geometry(_p(sz), _p(sp), _p(org), _p(d), _p(f), _p(osz), _p(osp), _p(oorg))
    return osz, osp, oorg


def bspline3(u):
    return lib().orc_bspline3(float(u))


def bspline3_derivative(u):
    return lib().orc_bspline3_derivative(float(u))


def mt_sequence(seed, n, skip=0):
    """MT19937 32-bit outputs (GetIntegerVariate) after `skip` draws from SetSeed(seed)."""
    out = np.zeros(int(n), np.uint32)
    lib().orc_mt_sequence(int(seed) & 0xFFFFFFFF, int(skip), _p(out), out.size)
    return out


def mt_normals(seed, n):
    """GetNormalVariate() sequence from SetSeed(seed)."""
    out = np.zeros(int(n), np.float64)
    lib().orc_mt_normals(int(seed) & 0xFFFFFFFF, _p(out), out.size)
    return out


def sample_points(strategy, size_xyz, spacing, origin, direction, percentage, seed):
    """ImageRegistrationMethodv4::SetMetricSamplePoints (strategy 1 REGULAR, 2 RANDOM)
    over a virtual domain; float32 points, shape (n, 3)."""
    size = np.ascontiguousarray(np.asarray(size_xyz, np.int64))
    V = int(np.prod(size))
    cap = V
    geo = np.ascontiguousarray(np.concatenate([np.asarray(spacing, np.float64), np.asarray(origin, np.float64),
                                               np.asarray(direction, np.float64).reshape(9)]))
    out = np.zeros((max(cap, 1), 3), np.float32)
    n = np.zeros(1, np.int64)
    rc = lib().orc_sample_points(int(strategy), _p(size), _p(geo), float(percentage), int(seed), _p(out), cap,
                                 _p(n))
    if rc != 0:
        raise ValueError(f"orc_sample_points status {rc}")
    return out[:int(n[0])].copy()
