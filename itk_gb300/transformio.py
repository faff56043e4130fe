"""Transform files in the reference's text format ("#Insight Transform File V1.0").

Mirrors itk::TransformFileWriter / TransformFileReader with the text IO
(Modules/IO/TransformInsightLegacy/src/itkTxtTransformIO.cxx:119-310): one
"#Transform k" block per transform with its type string
(Transform::GetTransformTypeAsString, Core/Transform/include/itkTransform.hxx:40-47:
class name, parameter type, input and output dimension), "Parameters:" and
"FixedParameters:" lines; a CompositeTransform is written as its type line
followed by its components in queue order.  Numbers are written as the
reference's NumberToString writes them (Core/Common/src/itkNumberToString.cxx:
the shortest string that reads back to the same double, in ECMAScript's
Number-to-String layout).
"""
from __future__ import annotations

import math

import numpy as np

from .transforms import AffineTransform, BSplineTransform, CompositeTransform, DisplacementFieldTransform

HEADER = "#Insight Transform File V1.0"
_TYPES = {
    "AffineTransform_double_3_3": AffineTransform,
    "BSplineTransform_double_3_3": BSplineTransform,
    "CompositeTransform_double_3_3": CompositeTransform,
    "DisplacementFieldTransform_double_3_3": DisplacementFieldTransform,
}


def number_to_string(x: float) -> str:
    """Shortest round-trip decimal in ECMAScript's layout: plain digits for decimal
    exponents in (-6, 21], otherwise d.ddde+n / d.ddde-n; 0 and -0 as "0"."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    if x == 0.0:
        return "0"
    sign = "-" if x < 0 else ""
    r = repr(abs(x))  # shortest round-trip digits
    mant, _, exp = r.partition("e")
    e = int(exp) if exp else 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    # value = 0.<digits> * 10^n
    lead_zeros = len(ip + fp) - len((ip + fp).lstrip("0"))
    n = len(ip) - lead_zeros + e
    digits = digits.rstrip("0") or "0"
    k = len(digits)
    if k <= n <= 21:
        s = digits + "0" * (n - k)
    elif 0 < n <= 21:
        s = digits[:n] + "." + digits[n:]
    elif -6 < n <= 0:
        s = "0." + "0" * (-n) + digits
    else:
        ex = n - 1
        es = ("+" if ex >= 0 else "-") + str(abs(ex))
        s = (digits if k == 1 else digits[0] + "." + digits[1:]) + "e" + es
    return sign + s


def _type_string(t) -> str:
    if isinstance(t, CompositeTransform):
        return "CompositeTransform_double_3_3"
    if isinstance(t, BSplineTransform):
        return "BSplineTransform_double_3_3"
    if isinstance(t, AffineTransform):
        return "AffineTransform_double_3_3"
    if isinstance(t, DisplacementFieldTransform):
        return "DisplacementFieldTransform_double_3_3"
    raise TypeError(f"no transform file type for {type(t).__name__}")


def _vector(v) -> str:
    return " ".join(number_to_string(x) for x in np.asarray(v, np.float64).reshape(-1))


def transform_to_text(transform) -> str:
    """TransformFileWriter's text for one transform (a composite: its components follow)."""
    items = [transform]
    if isinstance(transform, CompositeTransform):
        items = [transform] + [transform.GetNthTransform(i) for i in range(transform.GetNumberOfTransforms())]
    out = [HEADER]
    for k, t in enumerate(items):
        out.append(f"#Transform {k}")
        out.append(f"Transform: {_type_string(t)}")
        if isinstance(t, CompositeTransform):
            continue
        out.append("Parameters: " + _vector(t.GetParameters()))
        out.append("FixedParameters: " + _vector(t.GetFixedParameters()))
    return "\n".join(out) + "\n"


def WriteTransform(transform, filename: str):
    with open(filename, "w") as f:
        f.write(transform_to_text(transform))


def transforms_from_text(text: str):
    """TransformFileReader's list: every "Transform:" line makes a transform; its
    "FixedParameters:" are set before its "Parameters:" whichever comes first."""
    out = []
    cur, pending_params = None, None
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        if ":" not in line:
            raise ValueError("Tags must be delimited by :")
        name, value = (s.strip() for s in line.split(":", 1))
        if name == "Transform":
            if value not in _TYPES:
                raise ValueError(f"Could not create an instance of {value}")
            cur = _TYPES[value]()
            pending_params = None
            out.append(cur)
        elif name in ("Parameters", "FixedParameters"):
            if cur is None:
                raise ValueError(f"{name} before any Transform")
            vals = np.array([float(v) for v in value.split()], np.float64)
            if name == "FixedParameters":
                cur.SetFixedParameters(vals)
                if pending_params is not None:
                    cur.SetParameters(pending_params)
                    pending_params = None
            elif isinstance(cur, (BSplineTransform, DisplacementFieldTransform)) and \
                    cur.GetNumberOfParameters() != vals.size:
                pending_params = vals  # the grid comes with the fixed parameters
            else:
                cur.SetParameters(vals)
    return out


def ReadTransform(filename: str):
    """The transform in a file; a composite file gives the CompositeTransform with its components."""
    with open(filename) as f:
        ts = transforms_from_text(f.read())
    if not ts:
        raise ValueError("no transform in file")
    if isinstance(ts[0], CompositeTransform):
        c = ts[0]
        for t in ts[1:]:
            c.AddTransform(t)
        return c
    return ts[0]
